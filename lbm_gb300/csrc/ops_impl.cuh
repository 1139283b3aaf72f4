// Launcher bodies for one storage type S; included by step_fp64.cu, step_fp32.cu, step_fp16.cu
// and step_bf16.cu, each of which defines LBMG_STORE and LBMG_OPS_NAME before including it.
#pragma once

#include <algorithm>
#include <mutex>

#include "ops.cuh"
#include "state_kernels.cuh"
#include "adjoint.cuh"

namespace lbmg {
namespace {

inline dim3 cell_grid(const Geom& g)
{
    return dim3(static_cast<unsigned>((g.xl + kBlockX - 1) / kBlockX), static_cast<unsigned>(g.yl),
                static_cast<unsigned>(g.zl));
}

constexpr int kMaxDevices = 64;

inline unsigned linear_blocks(size_t n, unsigned threads)
{
    const size_t b = (n + threads - 1) / threads;
    return static_cast<unsigned>(b < 65535u * 16u ? (b > 0 ? b : 1) : 65535u * 16u);
}

// tau with its reciprocal pair for the FP64 collision's divisions (divrn.cuh)
inline DivRN tau_div(const DomainDev& d) { return make_div_rn(d.tau, 1.0 / d.tau); }

template <class L, class S>
StepParams<S> step_params(const DomainDev& d)
{
    StepParams<S> p;
    p.pop = static_cast<S*>(d.pop);
    p.flag = d.flag;
    p.link = d.link;
    p.bc = d.bc;
    p.edge = d.edge;
    p.n_edge = d.n_edge;
    p.ltab = d.ltab;
    p.wmask = d.wmask;
    p.profile = d.profile;
    p.g = d.g;
    p.err = d.err;
    p.mon = nullptr;
    p.rec = nullptr;
    p.tau = tau_div(d);
    p.omega = static_cast<float>(1.0 / d.tau);
    return p;
}

// Programmatic dependent launch of the kernels that run back to back in the time loop (the step
// and the adjoint step): their blocks may become resident while the previous kernel in the stream
// finishes and wait at their top (grid_dep_wait) for it to complete, which hides the launch gap
// between consecutive steps. LBMG_PDL 0 launches them plainly (tuning builds).
#ifndef LBMG_PDL
#define LBMG_PDL 1
#endif
template <class... KArgs, class... Args>
inline void launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                           const Args&... args)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = LBMG_PDL ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);  // a failure is left for cudaGetLastError
}

template <int Q, class S>
struct Launch {
    using L = Lattice<Q>;

    static void init(const DomainDev& d, cudaStream_t s)
    {
        init_kernel<L, S><<<linear_blocks(Q * d.g.PS, 256), 256, 0, s>>>(static_cast<S*>(d.pop), d.g.PS);
    }

    static void classify(const DomainDev& d, cudaStream_t s)
    {
        classify_kernel<L><<<cell_grid(d.g), kBlockX, 0, s>>>(d.flag, d.link, d.bc, d.g, Store<S>::kShifted);
    }

    static void side_passes(const DomainDev& d, long long k, cudaStream_t s)
    {
        const int copy = static_cast<int>(k & 1);
        S* pop = static_cast<S*>(d.pop);
        if (d.n_gf > 0)
            ghost_fluid_kernel<L, S><<<(d.n_gf + 127) / 128, 128, 0, s>>>(
                pop, d.flag, d.g, tau_div(d), d.gf_xyz, d.gf_pop, d.n_gf, copy);
        if (d.n_fs > 0)
            free_slip_kernel<L, S><<<(d.n_fs + 127) / 128, 128, 0, s>>>(
                pop, d.flag, d.g, d.fs_link, d.n_fs, copy, d.gf_pop, d.n_gf, copy);
    }

    static void step(const DomainDev& d, long long t, int mon_set, double* prev_out, void* rec, cudaStream_t s)
    {
        StepParams<S> p = step_params<L, S>(d);
        p.mon = mon_set >= 0 ? d.mon + 4 * kMonBuckets * mon_set : nullptr;
        p.mon_prev = mon_set >= 0 && prev_out ? d.mon + 4 * kMonBuckets * (1 - mon_set) : nullptr;
        p.mon_prev_out = prev_out;
        p.rec = static_cast<typename Store<S>::C*>(rec);
        const int nseg_x = (d.g.xl + kRowCells - 1) / kRowCells;
        const int nseg = nseg_x * d.g.yl * d.g.zl;
        constexpr int kSegs = segs<S>();
        const int row_blocks = (nseg + kSegs - 1) / kSegs;
        const int n_edge_blocks = (d.n_edge + kRowCells - 1) / kRowCells;
        const long long total = static_cast<long long>(n_edge_blocks) + row_blocks;
        // An edge block runs several times longer than a row block (gathers, handler lookups):
        // spread over the whole grid, the last ones would still run after every row block has
        // finished. They are spread over the first kEdgeSpan of the grid instead.
        const long long span = std::max<long long>(n_edge_blocks, static_cast<long long>(total * kEdgeSpan));
        const int edge_stride = n_edge_blocks > 0 ? static_cast<int>(std::max<long long>(1, span / n_edge_blocks)) : 1;
        const unsigned blocks = static_cast<unsigned>(total);
        const FastDiv fes = make_fastdiv(static_cast<uint32_t>(edge_stride));
        const FastDiv fx = make_fastdiv(static_cast<uint32_t>(nseg_x));
        const FastDiv fy = make_fastdiv(static_cast<uint32_t>(d.g.yl));
        constexpr size_t smem = row_smem_bytes<L, S>();
        if constexpr (smem > 48 * 1024) {  // only with more than one segment per block
            // the opt-in applies to the current device: once per device and kernel set
            static std::mutex m;
            static bool opted_in[kMaxDevices] = {};
            int dev = 0;
            cudaGetDevice(&dev);
            std::lock_guard<std::mutex> lock(m);
            if (dev >= 0 && dev < kMaxDevices && !opted_in[dev]) {
                for (auto k : {step_kernel<L, S, true, false, true>, step_kernel<L, S, false, false, true>,
                               step_kernel<L, S, true, true, true>, step_kernel<L, S, false, true, true>,
                               step_kernel<L, S, true, false, false>, step_kernel<L, S, false, false, false>})
                    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
                opted_in[dev] = true;
            }
        }
        const bool instr = mon_set >= 0 || rec != nullptr;
        // domains without handler cells (periodic boxes) take plain steps without the handler path:
        // its code alone slowed the FP32 periodic box by 7% (the instrumented steps keep it)
        const bool links = d.links != 0;
        auto* k = (t & 1) ? (instr   ? step_kernel<L, S, true, true, true>
                             : links ? step_kernel<L, S, true, false, true>
                                     : step_kernel<L, S, true, false, false>)
                          : (instr   ? step_kernel<L, S, false, true, true>
                             : links ? step_kernel<L, S, false, false, true>
                                     : step_kernel<L, S, false, false, false>);
        launch_chained(k, dim3(blocks), dim3(kRowCells), smem, s, p, n_edge_blocks, fes, nseg, fx, fy);
        side_passes(d, t, s);
    }

    static void gather(const DomainDev& d, long long k, double* out, cudaStream_t s)
    {
        const size_t ng = static_cast<size_t>(d.g.xl + 2) * (d.g.yl + 2) * (d.g.zl + 2);
        gather_kernel<L, S><<<linear_blocks(ng, 256), 256, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), out);
        if (d.n_gf > 0)
            ghost_fluid_io_kernel<L><<<(d.n_gf + 127) / 128, 128, 0, s>>>(
                d.g, d.gf_xyz, d.gf_pop, d.n_gf, static_cast<int>(k & 1), out, 1);
    }

    static void scatter(const DomainDev& d, long long k, const double* in, cudaStream_t s)
    {
        S* pop = static_cast<S*>(d.pop);
        scatter_kernel<L, S><<<cell_grid(d.g), kBlockX, 0, s>>>(pop, d.flag, d.g,
                                                                static_cast<int>(k & 1), in);
        if (d.n_gf > 0) {
            const int copy = static_cast<int>(k & 1);
            ghost_fluid_io_kernel<L><<<(d.n_gf + 127) / 128, 128, 0, s>>>(
                d.g, d.gf_xyz, d.gf_pop, d.n_gf, copy, const_cast<double*>(in), 0);
            ghost_fluid_slots_kernel<L, S><<<(d.n_gf + 127) / 128, 128, 0, s>>>(
                pop, d.flag, d.g, d.gf_xyz, d.gf_pop, d.n_gf, copy);
        }
    }

    static void moments(const DomainDev& d, long long k, double* rho, double* u, cudaStream_t s)
    {
        moments_kernel<L, S><<<cell_grid(d.g), kBlockX, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), rho, u);
    }

    static void monitor_fold(const DomainDev& d, int mon_set, double* out, cudaStream_t s)
    {
        monitor_fold_kernel<<<1, kMonFoldThreads, 0, s>>>(d.mon + 4 * kMonBuckets * mon_set, out);
    }

    static void gather_range(const DomainDev& d, long long k, size_t r0, size_t r1, double* out, cudaStream_t s)
    {
        gather_range_kernel<L, S><<<linear_blocks(r1 - r0, 256), 256, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), r0, r1, out);
    }

    static void scatter_range(const DomainDev& d, long long k, size_t r0, size_t r1, const double* in, cudaStream_t s)
    {
        scatter_range_kernel<L, S><<<linear_blocks(r1 - r0, 256), 256, 0, s>>>(
            static_cast<S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), r0, r1, in);
    }

    static void moments_range(const DomainDev& d, long long k, size_t n0, size_t n1, double* rho, double* u,
                              cudaStream_t s)
    {
        moments_range_kernel<L, S><<<linear_blocks(n1 - n0, 256), 256, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), n0, n1, rho, u);
    }

    static void ghost_fluid_slots(const DomainDev& d, long long k, cudaStream_t s)
    {
        if (d.n_gf > 0)
            ghost_fluid_slots_kernel<L, S><<<(d.n_gf + 127) / 128, 128, 0, s>>>(
                static_cast<S*>(d.pop), d.flag, d.g, d.gf_xyz, d.gf_pop, d.n_gf, static_cast<int>(k & 1));
    }

    static void reduce(const DomainDev& d, long long k, double* partials, int nblocks,
                       double* out, cudaStream_t s)
    {
        reduce_kernel<L, S><<<nblocks, kReduceThreads, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), partials);
        reduce_final_kernel<<<1, 32, 0, s>>>(partials, nblocks, out);
    }

    using T = typename Store<S>::C;

    static void adj_terminal(const DomainDev& d, const void* rec, void* mu_out, Box box, cudaStream_t s)
    {
        adjoint_terminal_kernel<L, T><<<cell_grid(d.g), kBlockX, 0, s>>>(
            d.flag, d.g, static_cast<T>(1.0 / d.tau), static_cast<const T*>(rec), box, static_cast<T*>(mu_out));
    }

    static void adj_step(const DomainDev& d, const void* mu_in, void* mu_out, const void* rec, int bc_terms,
                         int write_mu, double* grad_inflow, double* grad_wall, cudaStream_t s)
    {
        AdjParams<T> a;
        a.flag = d.flag;
        a.link = d.link;
        a.ltab = d.ltab;
        a.bc = d.bc;
        a.profile = d.profile;
        a.g = d.g;
        a.omega = static_cast<T>(1.0 / d.tau);
        a.mu_in = static_cast<const T*>(mu_in);
        a.mu_out = static_cast<T*>(mu_out);
        a.rec = static_cast<const T*>(rec);
        a.bc_terms = bc_terms;
        a.write_mu = write_mu;
        a.grad_inflow = grad_inflow;
        a.grad_wall = grad_wall;
        launch_chained(adjoint_step_kernel<L, T>, cell_grid(d.g), dim3(kBlockX), 0, s, a);
    }

    static void objective_ke(const DomainDev& d, long long k, Box box, double* partials, int nblocks,
                             double* out, cudaStream_t s)
    {
        objective_ke_kernel<L, S><<<nblocks, kReduceThreads, 0, s>>>(
            static_cast<const S*>(d.pop), d.flag, d.g, static_cast<int>(k & 1), box, partials);
        reduce_final_kernel<<<1, 32, 0, s>>>(partials, nblocks, out);
    }

    static void link_table(const DomainDev& d, LinkRecord* ltab, int* counter, int capacity, cudaStream_t s)
    {
        link_table_kernel<L><<<cell_grid(d.g), kBlockX, 0, s>>>(d.flag, d.link, d.bc, d.profile, d.g, ltab, counter,
                                                                 capacity);
    }

    static void warp_mask(const DomainDev& d, uint8_t* out, cudaStream_t s)
    {
        const int nseg_x = (d.g.xl + kRowCells - 1) / kRowCells;
        warp_mask_kernel<<<dim3(static_cast<unsigned>(nseg_x), static_cast<unsigned>(d.g.yl),
                                static_cast<unsigned>(d.g.zl)),
                           kRowCells, 0, s>>>(d.flag, d.g, nseg_x, out);
    }

    static const KernelOps* table()
    {
        static const KernelOps t = {&init,         &classify,      &step,          &monitor_fold, &gather,
                                    &scatter,      &moments,       &gather_range,  &scatter_range,
                                    &moments_range, &ghost_fluid_slots, &reduce,   sizeof(T),
                                    &adj_terminal, &adj_step,      &link_table,    &objective_ke,
                                    &warp_mask,    kRowCells};
        return &t;
    }
};

}  // namespace

const KernelOps* LBMG_OPS_NAME(int q)
{
    switch (q) {
    case 15: return Launch<15, LBMG_STORE>::table();
    case 19: return Launch<19, LBMG_STORE>::table();
    case 27: return Launch<27, LBMG_STORE>::table();
    default: return nullptr;
    }
}

}  // namespace lbmg
