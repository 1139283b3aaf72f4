// Host side of the C ABI declared in include/lbm_gb300.h.
//
// A handle keeps the geometry as a host byte map in the device layout (one byte per cell:
// fluid, ghost-fluid or handler id), the handler table, and the device state. Geometry calls
// only touch the host map; the next call that needs the device state uploads it, classifies the
// fluid cells, rebuilds the side-pass lists and, when the populations are no longer the initial
// ones, carries them across the change (read back with the old geometry, written with the new).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "domain.cuh"
#include "lattice.cuh"
#include "ops.cuh"

using namespace lbmg;

namespace {

// Slots of the device ring that holds per-step monitor results until their copy to the host (one
// copy per kMonRing steps).
constexpr int kMonRing = 1024;
// Largest staging slot of the chunked host transfers (two slots per handle, allocated on the
// first transfer and kept).
constexpr size_t kStageSlotBytes = size_t(32) << 20;

thread_local std::string g_create_error;

struct CudaError : std::runtime_error {
    int code;
    CudaError(const std::string& what, int c) : std::runtime_error(what), code(c) {}
};
struct ArgError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        const int code = (e == cudaErrorMemoryAllocation) ? LBM_ERR_OOM : LBM_ERR_CUDA;
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), code);
    }
}

size_t store_bytes(int precision) { return precision == LBM_FP64 ? 8 : (precision == LBM_FP32 ? 4 : 2); }

// Lattice velocity component, host side.
int lat_c(int q, int Q, int d)
{
    switch (Q) {
    case 15: return Lattice<15>::c(q, d);
    case 19: return Lattice<19>::c(q, d);
    default: return Lattice<27>::c(q, d);
    }
}
double lat_w(int q, int Q)
{
    switch (Q) {
    case 15: return Lattice<15>::w(q);
    case 19: return Lattice<19>::w(q);
    default: return Lattice<27>::w(q);
    }
}
int lat_velocity_index(int Q, int u, int v, int w)
{
    switch (Q) {
    case 15: return Lattice<15>::velocity_index(u, v, w);
    case 19: return Lattice<19>::velocity_index(u, v, w);
    default: return Lattice<27>::velocity_index(u, v, w);
    }
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void alloc(size_t count, const char* what)
    {
        release();
        if (count == 0) return;
        const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            // a failed allocation is not a sticky error: clear it, so that a later
            // cudaGetLastError of this thread does not report it against another call
            cudaGetLastError();
            check(e, what);
        }
        n = count;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

}  // namespace

// Checkpoints of a gradient run (lbm_adjoint_forward .. lbm_adjoint_backward), and the backward's
// workspace: allocated by the first lbm_adjoint_backward of a run's geometry and checkpoint
// interval and kept for the next calls, so that repeated gradients cost no allocation. A run with
// a checkpoint every step (k = 1) keeps the forward's per-step records instead of state copies:
// the backward then recomputes nothing and leaves the state alone.
struct AdjointRun {
    bool ready = false;
    bool resident = false;  // k = 1: rec holds the records of all n steps, written by the forward
    long long s0 = 0;  // steps done when the run started
    long long n = 0;   // steps of the run
    long long k = 0;   // steps between checkpoints
    std::vector<std::unique_ptr<DevBuf<unsigned char>>> ckpt;  // state after s0 + j*k steps
    DevBuf<unsigned char> mu[2];   // adjoint populations mu_t, mu_{t-1}
    DevBuf<unsigned char> rec;     // the recorded mass and momentum of a segment's k steps (of
                                   // all n steps when resident)
    DevBuf<unsigned char> rec2;    // a second segment record: the recompute of one segment
                                   // overlaps the adjoint steps of the next
    DevBuf<unsigned char> backup;  // the state the forward run left
    DevBuf<double> gin, gwall;     // gradients (inflow cells, wall handlers)
    // the recompute stream and its events (record buffer b filled / read), created on first use
    cudaStream_t rstream = nullptr;
    cudaEvent_t filled[2] = {nullptr, nullptr};
    cudaEvent_t drained[2] = {nullptr, nullptr};
    void release_workspace()
    {
        mu[0].release(); mu[1].release(); rec.release(); rec2.release(); backup.release(); gin.release();
        gwall.release();
    }
    ~AdjointRun()
    {
        for (int b = 0; b < 2; ++b) {
            if (filled[b]) cudaEventDestroy(filled[b]);
            if (drained[b]) cudaEventDestroy(drained[b]);
        }
        if (rstream) cudaStreamDestroy(rstream);
    }
};

struct lbm_domain {
    DomainDev dev{};
    AdjointRun adj;
    const KernelOps* ops = nullptr;
    cudaStream_t stream = nullptr;
    int Q = 0;
    int precision = 0;
    int device = 0;         // device current at lbm_create
    size_t ng = 0;         // cells incl. ghost layer
    size_t n_interior = 0;
    uint64_t fluid_cells = 0;

    std::vector<uint8_t> hmap;                  // PS bytes, device layout
    std::vector<BcEntry> bcs;                   // handler h at index h-1
    std::vector<std::vector<double>> profiles;  // per handler: empty or 3*ng doubles

    bool geom_dirty = true;
    bool state_custom = false;
    long long steps = 0;

    DevBuf<unsigned char> pop;
    DevBuf<uint8_t> flag;
    DevBuf<BcEntry> bc;
    DevBuf<double> profile;
    DevBuf<int> gf_xyz;
    DevBuf<double> gf_pop;
    DevBuf<int4> fs_link;
    DevBuf<double> red;  // 4 * kReduceBlocks partials + 4 totals
    DevBuf<uint2> link;     // per-cell link words and LinkRecord rows
    DevBuf<int> edge;       // kFluidEdge cells
    DevBuf<LinkRecord> ltab;  // LinkRecords (shifted storage)
    DevBuf<uint8_t> wmask;    // the step kernel's per-segment warp mask
    DevBuf<int> errword;    // device error word, a list counter
    DevBuf<double> mon;     // step monitor accumulators
    DevBuf<double> mon_ring;  // per-step monitor results, kMonRing slots of 4 doubles
    std::vector<int> gf_host;  // x, y, z of every ghost-fluid side-pass cell (as gf_xyz)

    // Staging of the chunked host transfers (populations, moments): two device slots that take
    // turns, so that the copy of one chunk (on copy_stream) overlaps the kernel of the other (on
    // stream). Allocated by the first transfer and kept with the handle.
    DevBuf<unsigned char> stage;
    size_t stage_slot = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_ready[2] = {nullptr, nullptr};  // slot filled (kernel done / upload done)
    cudaEvent_t ev_free[2] = {nullptr, nullptr};   // slot consumed (download done / kernel done)
    cudaEvent_t ev_start = nullptr;

    std::string err;

    ~lbm_domain()
    {
        pop.release(); flag.release(); bc.release(); profile.release();
        gf_xyz.release(); gf_pop.release(); fs_link.release(); red.release(); link.release(); edge.release(); errword.release(); mon.release(); mon_ring.release();
        stage.release();
        for (int k = 0; k < 2; ++k) {
            if (ev_ready[k]) cudaEventDestroy(ev_ready[k]);
            if (ev_free[k]) cudaEventDestroy(ev_free[k]);
        }
        if (ev_start) cudaEventDestroy(ev_start);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }

    size_t layout_index(int x, int y, int z) const
    {
        return static_cast<size_t>(kXOff + x) +
               static_cast<size_t>(dev.g.XS) *
                   (static_cast<size_t>(y) + static_cast<size_t>(dev.g.YS) * static_cast<size_t>(z));
    }
    size_t ref_index(int x, int y, int z) const
    {
        return static_cast<size_t>(x) +
               static_cast<size_t>(dev.g.xl + 2) *
                   (static_cast<size_t>(y) + static_cast<size_t>(dev.g.yl + 2) * static_cast<size_t>(z));
    }
    bool interior(int x, int y, int z) const
    {
        return x >= 1 && x <= dev.g.xl && y >= 1 && y <= dev.g.yl && z >= 1 && z <= dev.g.zl;
    }
    bool on_periodic_ghost(int x, int y, int z) const
    {
        const Geom& g = dev.g;
        return ((g.per & 1) && (x == 0 || x == g.xl + 1)) || ((g.per & 2) && (y == 0 || y == g.yl + 1)) ||
               ((g.per & 4) && (z == 0 || z == g.zl + 1));
    }
    void wrap(int& x, int& y, int& z) const
    {
        const Geom& g = dev.g;
        auto w = [](int v, int l, bool p) { return p ? (v < 1 ? v + l : (v > l ? v - l : v)) : v; };
        x = w(x, g.xl, g.per & 1);
        y = w(y, g.yl, g.per & 2);
        z = w(z, g.zl, g.per & 4);
    }
    uint8_t hm(int x, int y, int z) const { return hmap[layout_index(x, y, z)]; }

    void finalize();
    void build_side_lists();
    void build_edge_list();
    void build_link_table();
    void check_device_error();
    void ensure_staging();
    void upload_state(const double* f);
    void download_state(double* f);
    void download_moments(double* rho, double* u);
};

namespace {

__global__ void scale_kernel(double* v, size_t n, double a)
{
    for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<size_t>(gridDim.x) * blockDim.x)
        v[k] *= a;
}

void scale_doubles(double* v, size_t n, double a, cudaStream_t s)
{
    if (n == 0) return;
    const size_t blocks = std::min<size_t>((n + 255) / 256, 4096);
    scale_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(v, n, a);
}

// Appends the layout index of every kFluidEdge cell (the host sorts the list afterwards).
__global__ void collect_edges_kernel(const uint8_t* flag, Geom g, int* list, int* count, int cap)
{
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = kXOff + x + g.XS * (y + g.YS * z);
    if (flag[i] != kFluidEdge) return;
    const int k = atomicAdd(count, 1);
    if (k < cap) list[k] = i;
}

}  // namespace

void lbm_domain::build_edge_list()
{
    const Geom& g = dev.g;
    edge.release();
    const dim3 grid(static_cast<unsigned>((g.xl + kBlockX - 1) / kBlockX), static_cast<unsigned>(g.yl),
                    static_cast<unsigned>(g.zl));
    int* counter = errword.p + 1;
    int n = 0;
    check(cudaMemsetAsync(counter, 0, sizeof(int), stream), "edge count reset");
    collect_edges_kernel<<<grid, kBlockX, 0, stream>>>(flag.p, g, nullptr, counter, 0);
    check(cudaMemcpyAsync(&n, counter, sizeof(int), cudaMemcpyDeviceToHost, stream), "edge count");
    check(cudaStreamSynchronize(stream), "edge count");
    if (n > 0) {
        edge.alloc(static_cast<size_t>(n), "cudaMalloc(edge list)");
        check(cudaMemsetAsync(counter, 0, sizeof(int), stream), "edge count reset");
        collect_edges_kernel<<<grid, kBlockX, 0, stream>>>(flag.p, g, edge.p, counter, n);
        std::vector<int> h(static_cast<size_t>(n));
        check(cudaMemcpyAsync(h.data(), edge.p, h.size() * sizeof(int), cudaMemcpyDeviceToHost, stream),
              "edge list");
        check(cudaStreamSynchronize(stream), "edge list");
        std::sort(h.begin(), h.end());  // neighbouring edge cells in neighbouring threads
        check(cudaMemcpyAsync(edge.p, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, stream),
              "edge list upload");
        check(cudaStreamSynchronize(stream), "edge list upload");
    }
    dev.edge = edge.p;
    dev.n_edge = n;
}

void lbm_domain::build_link_table()
{
    int* counter = errword.p + 1;
    int n = 0;
    check(cudaMemsetAsync(counter, 0, sizeof(int), stream), "link record count reset");
    ops->link_table(dev, nullptr, counter, 0, stream);
    check(cudaMemcpyAsync(&n, counter, sizeof(int), cudaMemcpyDeviceToHost, stream), "link record count");
    check(cudaStreamSynchronize(stream), "link record count");
    if (n > 0) {
        if (ltab.n < static_cast<size_t>(n)) ltab.alloc(static_cast<size_t>(n), "cudaMalloc(link records)");
        check(cudaMemsetAsync(counter, 0, sizeof(int), stream), "link record count reset");
        ops->link_table(dev, ltab.p, counter, n, stream);  // classify left every row at kNoRecord
        check(cudaGetLastError(), "link record kernel");
    }
    dev.ltab = n > 0 ? ltab.p : nullptr;
}

void lbm_domain::check_device_error()
{
    int e = 0;
    check(cudaMemcpyAsync(&e, errword.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "read device error word");
    check(cudaStreamSynchronize(stream), "read device error word");
    if (e != 0) {
        check(cudaMemsetAsync(errword.p, 0, sizeof(int), stream), "clear device error word");
        check(cudaStreamSynchronize(stream), "clear device error word");
        throw CudaError("a bounded wait inside the step kernel gave up; the results of the steps since the "
                        "last check are not valid", LBM_ERR_CUDA);
    }
}

// Ghost-fluid cells adjacent to interior fluid (or used as a free-slip source) and the
// free-slip links, from the host map.
void lbm_domain::build_side_lists()
{
    const Geom& g = dev.g;
    // earlier work on the stream may still read the lists released below
    check(cudaStreamSynchronize(stream), "side-list rebuild");
    std::vector<int> gxyz;
    std::unordered_map<size_t, int> gf_index;  // layout index -> position in the ghost-fluid list
    auto gf_add = [&](int x, int y, int z) -> int {
        const auto it = gf_index.emplace(layout_index(x, y, z), static_cast<int>(gxyz.size() / 3));
        if (it.second) {
            gxyz.push_back(x); gxyz.push_back(y); gxyz.push_back(z);
        }
        return it.first->second;
    };
    auto is_fluid_h = [&](int x, int y, int z) {
        const uint8_t v = hm(x, y, z);
        return v < kFirstHandler && !on_periodic_ghost(x, y, z);  // interior fluid or ghost fluid
    };
    auto interior_fluid_h = [&](int x, int y, int z) { return interior(x, y, z) && hm(x, y, z) == 0; };

    // ghost-fluid cells with an interior fluid neighbour
    for (int z = 0; z <= g.zl + 1; ++z)
        for (int y = 0; y <= g.yl + 1; ++y)
            for (int x = 0; x <= g.xl + 1; ++x) {
                if (interior(x, y, z) || on_periodic_ghost(x, y, z)) continue;
                if (hm(x, y, z) != kGhostFluid) continue;
                bool adj = false;
                for (int q = 0; q < Q && !adj; ++q) {
                    int nx = x + lat_c(q, Q, 0), ny = y + lat_c(q, Q, 1), nz = z + lat_c(q, Q, 2);
                    wrap(nx, ny, nz);
                    if (interior_fluid_h(nx, ny, nz)) adj = true;
                }
                if (adj) gf_add(x, y, z);
            }

    // free-slip links (boundary.hpp:79-115)
    std::vector<int4> links;
    for (int z = 0; z <= g.zl + 1; ++z)
        for (int y = 0; y <= g.yl + 1; ++y)
            for (int x = 0; x <= g.xl + 1; ++x) {
                const uint8_t v = hm(x, y, z);
                if (v < kFirstHandler || on_periodic_ghost(x, y, z)) continue;
                if (bcs[v - kFirstHandler].type != kFreeSlip) continue;
                for (int q = 0; q < Q; ++q) {
                    const int dx = lat_c(q, Q, 0), dy = lat_c(q, Q, 1), dz = lat_c(q, Q, 2);
                    int nx = x + dx, ny = y + dy, nz = z + dz;
                    wrap(nx, ny, nz);
                    if (!interior_fluid_h(nx, ny, nz)) continue;
                    const int cand[6][3] = {{x + dx, y, z}, {x, y + dy, z}, {x, y, z + dz},
                                            {x, y + dy, z + dz}, {x + dx, y, z + dz}, {x + dx, y + dy, z}};
                    const int mir[6][3] = {{-dx, dy, dz}, {dx, -dy, dz}, {dx, dy, -dz},
                                           {dx, -dy, -dz}, {-dx, dy, -dz}, {-dx, -dy, dz}};
                    for (int k = 0; k < 6; ++k) {
                        int sx = cand[k][0], sy = cand[k][1], sz = cand[k][2];
                        wrap(sx, sy, sz);
                        if (!is_fluid_h(sx, sy, sz)) continue;
                        const int qs = lat_velocity_index(Q, mir[k][0], mir[k][1], mir[k][2]);
                        if (qs < 0 || qs >= Q) break;
                        int4 l;
                        l.x = static_cast<int>(layout_index(nx, ny, nz));
                        if (interior(sx, sy, sz)) {
                            int mx = sx + lat_c(qs, Q, 0), my = sy + lat_c(qs, Q, 1), mz = sz + lat_c(qs, Q, 2);
                            wrap(mx, my, mz);
                            l.y = q | (qs << 8);
                            l.z = static_cast<int>(layout_index(sx, sy, sz));
                            l.w = static_cast<int>(layout_index(mx, my, mz));
                        } else {
                            l.y = q | (qs << 8) | (1 << 16);
                            l.z = gf_add(sx, sy, sz);
                            l.w = 0;
                        }
                        links.push_back(l);
                        break;
                    }
                }
            }

    gf_xyz.release(); gf_pop.release(); fs_link.release();
    gf_host = gxyz;
    dev.n_gf = static_cast<int>(gxyz.size() / 3);
    dev.n_fs = static_cast<int>(links.size());
    if (dev.n_gf > 0) {
        gf_xyz.alloc(gxyz.size(), "cudaMalloc(ghost-fluid list)");
        check(cudaMemcpyAsync(gf_xyz.p, gxyz.data(), gxyz.size() * sizeof(int), cudaMemcpyHostToDevice, stream),
              "upload ghost-fluid list");
        gf_pop.alloc(static_cast<size_t>(2) * dev.n_gf * Q, "cudaMalloc(ghost-fluid populations)");
        std::vector<double> w(static_cast<size_t>(2) * dev.n_gf * Q);
        for (size_t k = 0; k < w.size(); ++k) w[k] = lat_w(static_cast<int>(k % Q), Q);
        check(cudaMemcpyAsync(gf_pop.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, stream),
              "init ghost-fluid populations");
        check(cudaStreamSynchronize(stream), "ghost-fluid setup");
    }
    if (dev.n_fs > 0) {
        fs_link.alloc(links.size(), "cudaMalloc(free-slip links)");
        check(cudaMemcpyAsync(fs_link.p, links.data(), links.size() * sizeof(int4), cudaMemcpyHostToDevice, stream),
              "upload free-slip links");
        check(cudaStreamSynchronize(stream), "free-slip setup");
    }
    dev.gf_xyz = gf_xyz.p;
    dev.gf_pop = gf_pop.p;
    dev.fs_link = fs_link.p;
}

void lbm_domain::finalize()
{
    if (!geom_dirty) return;
    adj.ready = false;
    adj.release_workspace();
    const Geom& g = dev.g;
    DevBuf<double> carry;
    if (state_custom) {
        // the current state, read with the geometry it was produced under
        carry.alloc(ng * Q, "cudaMalloc(state carry-over)");
        ops->gather(dev, steps, carry.p, stream);
    }
    check(cudaMemcpyAsync(flag.p, hmap.data(), hmap.size(), cudaMemcpyHostToDevice, stream), "upload flags");
    check(cudaMemcpyAsync(bc.p, bcs.data(), bcs.size() * sizeof(BcEntry), cudaMemcpyHostToDevice, stream),
          "upload handler table");
    ops->classify(dev, stream);  // reads the handler table (no-slip links)
    const size_t nseg = row_segments(g, ops->row_cells);
    if (wmask.n != nseg) wmask.alloc(nseg, "cudaMalloc(warp mask)");
    ops->warp_mask(dev, wmask.p, stream);
    dev.wmask = wmask.p;
    dev.links = std::any_of(hmap.begin(), hmap.end(), [](uint8_t v) { return v >= kFirstHandler; }) ? 1 : 0;
    // merged inflow profile in reference cell order
    bool any_profile = false;
    for (const auto& p : profiles) any_profile = any_profile || !p.empty();
    if (any_profile) {
        std::vector<double> merged(3 * ng, 0.0);
        for (int z = 0; z <= g.zl + 1; ++z)
            for (int y = 0; y <= g.yl + 1; ++y)
                for (int x = 0; x <= g.xl + 1; ++x) {
                    const uint8_t v = hm(x, y, z);
                    if (v < kFirstHandler) continue;
                    const auto& p = profiles[v - kFirstHandler];
                    if (p.empty()) continue;
                    const size_t r = ref_index(x, y, z);
                    merged[3 * r] = p[3 * r]; merged[3 * r + 1] = p[3 * r + 1]; merged[3 * r + 2] = p[3 * r + 2];
                }
        if (!profile.p) profile.alloc(3 * ng, "cudaMalloc(inflow profile)");
        check(cudaMemcpyAsync(profile.p, merged.data(), merged.size() * sizeof(double), cudaMemcpyHostToDevice, stream),
              "upload inflow profile");
        check(cudaStreamSynchronize(stream), "inflow profile");
    }
    dev.profile = profile.p;
    build_side_lists();
    build_edge_list();
    build_link_table();  // after the profile upload: inflow records hold the profile's values
    fluid_cells = 0;
    for (int z = 1; z <= g.zl; ++z)
        for (int y = 1; y <= g.yl; ++y) {
            const uint8_t* row = hmap.data() + layout_index(1, y, z);
            for (int x = 0; x < g.xl; ++x) fluid_cells += row[x] == 0;
        }
    if (state_custom) {
        ops->scatter(dev, steps, carry.p, stream);
        check(cudaStreamSynchronize(stream), "state carry-over");
        carry.release();
    }
    check(cudaGetLastError(), "finalize kernels");
    geom_dirty = false;
}

void lbm_domain::ensure_staging()
{
    if (stage.p) return;
    const size_t need = std::max(ng * static_cast<size_t>(Q), 4 * n_interior) * sizeof(double);
    stage_slot = std::min(kStageSlotBytes, (need + 255) / 256 * 256);
    stage_slot = std::max(stage_slot, static_cast<size_t>(Q) * sizeof(double) * 256);
    stage.alloc(2 * stage_slot, "cudaMalloc(transfer staging)");
    check(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(copy)");
    for (int k = 0; k < 2; ++k) {
        check(cudaEventCreateWithFlags(&ev_ready[k], cudaEventDisableTiming), "cudaEventCreate");
        check(cudaEventCreateWithFlags(&ev_free[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    check(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming), "cudaEventCreate");
}

// Host AoS FP64 field (reference cell order, all cells) -> state: chunk k is uploaded into slot
// k % 2 on the copy stream while the scatter of chunk k - 1 runs on the handle's stream.
void lbm_domain::upload_state(const double* f)
{
    ensure_staging();
    const size_t row = static_cast<size_t>(Q) * sizeof(double);
    const size_t rows = stage_slot / row;
    check(cudaEventRecord(ev_start, stream), "cudaEventRecord");
    check(cudaStreamWaitEvent(copy_stream, ev_start, 0), "cudaStreamWaitEvent");
    size_t k = 0;
    for (size_t r0 = 0; r0 < ng; r0 += rows, ++k) {
        const size_t r1 = std::min(ng, r0 + rows);
        const int slot = static_cast<int>(k & 1);
        double* buf = reinterpret_cast<double*>(stage.p + slot * stage_slot);
        if (k >= 2) check(cudaStreamWaitEvent(copy_stream, ev_free[slot], 0), "cudaStreamWaitEvent");
        check(cudaMemcpyAsync(buf, f + r0 * Q, (r1 - r0) * row, cudaMemcpyHostToDevice, copy_stream),
              "upload populations");
        check(cudaEventRecord(ev_ready[slot], copy_stream), "cudaEventRecord");
        check(cudaStreamWaitEvent(stream, ev_ready[slot], 0), "cudaStreamWaitEvent");
        ops->scatter_range(dev, steps, r0, r1, buf, stream);
        check(cudaEventRecord(ev_free[slot], stream), "cudaEventRecord");
    }
    check(cudaGetLastError(), "scatter kernel");
    if (dev.n_gf > 0) {
        // the ghost-fluid cells' side copy for this parity, then the slots they feed
        std::vector<double> h(static_cast<size_t>(dev.n_gf) * Q);
        for (int j = 0; j < dev.n_gf; ++j) {
            const size_t r = ref_index(gf_host[3 * j], gf_host[3 * j + 1], gf_host[3 * j + 2]);
            std::memcpy(h.data() + static_cast<size_t>(j) * Q, f + r * Q, row);
        }
        double* dst = gf_pop.p + static_cast<size_t>(steps & 1) * dev.n_gf * Q;
        check(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream),
              "upload ghost-fluid populations");
        ops->ghost_fluid_slots(dev, steps, stream);
        check(cudaGetLastError(), "ghost-fluid slots kernel");
    }
    check(cudaStreamSynchronize(stream), "set populations");
}

// State -> host AoS FP64 field: chunk k is gathered into slot k % 2 on the handle's stream while
// the download of chunk k - 1 runs on the copy stream.
void lbm_domain::download_state(double* f)
{
    ensure_staging();
    const size_t row = static_cast<size_t>(Q) * sizeof(double);
    const size_t rows = stage_slot / row;
    size_t k = 0;
    for (size_t r0 = 0; r0 < ng; r0 += rows, ++k) {
        const size_t r1 = std::min(ng, r0 + rows);
        const int slot = static_cast<int>(k & 1);
        double* buf = reinterpret_cast<double*>(stage.p + slot * stage_slot);
        if (k >= 2) check(cudaStreamWaitEvent(stream, ev_free[slot], 0), "cudaStreamWaitEvent");
        ops->gather_range(dev, steps, r0, r1, buf, stream);
        check(cudaEventRecord(ev_ready[slot], stream), "cudaEventRecord");
        check(cudaStreamWaitEvent(copy_stream, ev_ready[slot], 0), "cudaStreamWaitEvent");
        check(cudaMemcpyAsync(f + r0 * Q, buf, (r1 - r0) * row, cudaMemcpyDeviceToHost, copy_stream),
              "download populations");
        check(cudaEventRecord(ev_free[slot], copy_stream), "cudaEventRecord");
    }
    check(cudaGetLastError(), "gather kernel");
    std::vector<double> h(static_cast<size_t>(dev.n_gf) * Q);
    if (dev.n_gf > 0) {
        const double* src = gf_pop.p + static_cast<size_t>(steps & 1) * dev.n_gf * Q;
        check(cudaMemcpyAsync(h.data(), src, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream),
              "download ghost-fluid populations");
    }
    check(cudaStreamSynchronize(copy_stream), "get populations");
    check(cudaStreamSynchronize(stream), "get populations");
    for (int j = 0; j < dev.n_gf; ++j) {
        const size_t r = ref_index(gf_host[3 * j], gf_host[3 * j + 1], gf_host[3 * j + 2]);
        std::memcpy(f + r * Q, h.data() + static_cast<size_t>(j) * Q, row);
    }
}

// Interior density (and velocity) -> host, chunked as download_state.
void lbm_domain::download_moments(double* rho, double* u)
{
    ensure_staging();
    const size_t per = (u ? 4 : 1) * sizeof(double);
    const size_t cells = stage_slot / per;
    size_t k = 0;
    for (size_t n0 = 0; n0 < n_interior; n0 += cells, ++k) {
        const size_t n1 = std::min(n_interior, n0 + cells);
        const int slot = static_cast<int>(k & 1);
        double* buf = reinterpret_cast<double*>(stage.p + slot * stage_slot);
        double* ubuf = u ? buf + (n1 - n0) : nullptr;
        if (k >= 2) check(cudaStreamWaitEvent(stream, ev_free[slot], 0), "cudaStreamWaitEvent");
        ops->moments_range(dev, steps, n0, n1, buf, ubuf, stream);
        check(cudaEventRecord(ev_ready[slot], stream), "cudaEventRecord");
        check(cudaStreamWaitEvent(copy_stream, ev_ready[slot], 0), "cudaStreamWaitEvent");
        check(cudaMemcpyAsync(rho + n0, buf, (n1 - n0) * sizeof(double), cudaMemcpyDeviceToHost, copy_stream),
              "download density");
        if (u)
            check(cudaMemcpyAsync(u + 3 * n0, ubuf, 3 * (n1 - n0) * sizeof(double), cudaMemcpyDeviceToHost,
                                  copy_stream),
                  "download velocity");
        check(cudaEventRecord(ev_free[slot], copy_stream), "cudaEventRecord");
    }
    check(cudaGetLastError(), "moments kernel");
    check(cudaStreamSynchronize(copy_stream), "moments");
    check(cudaStreamSynchronize(stream), "moments");
}

namespace {

// Device scratch of lbm_moments_noalloc: density and velocity of up to kNoAllocMaxCells interior
// cells (4 doubles each, 8 MiB). It lives in every GPU that loads the library until the process
// exits, and all calls share it.
constexpr size_t kNoAllocMaxCells = 262144;
static __device__ __align__(256) double g_noalloc_moments[4 * kNoAllocMaxCells];

// Its device address, looked up once per device (with that device current) by the first
// lbm_moments_noalloc call on that device. The host-side name of the array is not a device
// address and is never handed to a kernel.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

double* noalloc_scratch(int device)
{
    if (device < 0 || device >= kNoAllocMaxDevices) throw ArgError("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        check(cudaGetSymbolAddress(&p, g_noalloc_moments), "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_ptr[device] = static_cast<double*>(p);
    }
    return g_noalloc_ptr[device];
}

// Makes the handle's device current for one call and restores the caller's device afterwards:
// the handle's stream, memory and kernels belong to the device that was current at lbm_create.
struct DeviceGuard {
    int prev = -1;
    int dev = -1;
    explicit DeviceGuard(int device) : dev(device)
    {
        if (device < 0) return;
        check(cudaGetDevice(&prev), "cudaGetDevice");
        if (prev != device) check(cudaSetDevice(device), "cudaSetDevice");
    }
    ~DeviceGuard()
    {
        if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
};

template <class F>
int guarded(lbm_domain* d, F&& f)
{
    if (!d) return LBM_ERR_ARG;
    try {
        DeviceGuard on_device(d->stream ? d->device : -1);  // lbm_create picks the device itself
        f();
        return LBM_OK;
    } catch (const CudaError& e) {
        d->err = e.what();
        return e.code;
    } catch (const ArgError& e) {
        d->err = e.what();
        return LBM_ERR_ARG;
    } catch (const StateError& e) {
        d->err = e.what();
        return LBM_ERR_STATE;
    } catch (const std::bad_alloc&) {
        d->err = "host allocation failed";
        return LBM_ERR_OOM;
    } catch (const std::exception& e) {
        d->err = e.what();
        return LBM_ERR_CUDA;
    } catch (...) {
        d->err = "unknown error";
        return LBM_ERR_CUDA;
    }
}

}  // namespace

extern "C" {

int lbm_create(lbm_domain** out, int q, int64_t xl, int64_t yl, int64_t zl, double tau, int precision)
{
    g_create_error.clear();
    if (!out) { g_create_error = "out is NULL"; return LBM_ERR_ARG; }
    *out = nullptr;
    if (q != 15 && q != 19 && q != 27) { g_create_error = "lattice model must be 15, 19 or 27"; return LBM_ERR_ARG; }
    if (!(tau > 0.5 && tau < 2.0)) { g_create_error = "tau must lie in (0.5, 2.0)"; return LBM_ERR_ARG; }
    if (xl < 1 || yl < 1 || zl < 1) { g_create_error = "domain lengths must be positive"; return LBM_ERR_ARG; }
    if (precision < LBM_FP64 || precision > LBM_BF16) { g_create_error = "unknown precision"; return LBM_ERR_ARG; }
    const int64_t XS = (xl + 2 + 31) / 32 * 32, YS = yl + 2, ZS = zl + 2;
    const int64_t cells = XS * YS * ZS;
    if (xl > (1 << 20) || yl > 65535 || zl > 65535 || cells + 1024 >= (int64_t(1) << 31)) {
        g_create_error = "domain too large (cell index must fit 31 bits, yl and zl <= 65535)";
        return LBM_ERR_ARG;
    }
    lbm_domain* d = nullptr;
    try {
        d = new lbm_domain();
    } catch (...) {
        g_create_error = "host allocation failed";
        return LBM_ERR_OOM;
    }
    const int rc = guarded(d, [&] {
        d->Q = q;
        d->precision = precision;
        Geom& g = d->dev.g;
        g.xl = static_cast<int>(xl); g.yl = static_cast<int>(yl); g.zl = static_cast<int>(zl);
        g.XS = static_cast<int>(XS); g.YS = static_cast<int>(YS); g.ZS = static_cast<int>(ZS);
        g.per = 0;
        g.PS = static_cast<size_t>((cells + 512 + 63) / 64 * 64);
        d->ng = static_cast<size_t>(xl + 2) * (yl + 2) * (zl + 2);
        d->n_interior = static_cast<size_t>(xl) * yl * zl;
        d->dev.q = q;
        d->dev.precision = precision;
        d->dev.tau = tau;
        switch (precision) {
        case LBM_FP64: d->ops = ops_fp64(q); break;
        case LBM_FP32: d->ops = ops_fp32(q); break;
        case LBM_FP16: d->ops = ops_fp16(q); break;
        default: d->ops = ops_bf16(q); break;
        }
        check(cudaGetDevice(&d->device), "cudaGetDevice");
        check(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        d->pop.alloc(static_cast<size_t>(q) * g.PS * store_bytes(precision), "cudaMalloc(populations)");
        d->flag.alloc(g.PS, "cudaMalloc(flags)");
        d->bc.alloc(kMaxHandlers, "cudaMalloc(handler table)");
        d->red.alloc(4 * kReduceBlocks + 4, "cudaMalloc(reduction scratch)");
        d->link.alloc(g.PS, "cudaMalloc(link words)");
        d->dev.link = d->link.p;
        d->errword.alloc(2, "cudaMalloc(error word)");  // error word, list counter
        check(cudaMemsetAsync(d->errword.p, 0, 2 * sizeof(int), d->stream), "clear error word");
        d->dev.err = d->errword.p;
        d->mon.alloc(2 * 4 * kMonBuckets, "cudaMalloc(step monitor)");  // two accumulator sets
        check(cudaMemsetAsync(d->mon.p, 0, d->mon.bytes(), d->stream), "clear step monitor");
        d->dev.mon = d->mon.p;
        d->mon_ring.alloc(4 * kMonRing, "cudaMalloc(step monitor ring)");
        d->dev.pop = d->pop.p;
        d->dev.flag = d->flag.p;
        d->dev.bc = d->bc.p;
        // host map: interior cells fluid, everything else ghost-fluid until a handler is set
        d->hmap.assign(g.PS, kGhostFluid);
        for (int z = 1; z <= g.zl; ++z)
            for (int y = 1; y <= g.yl; ++y)
                std::memset(d->hmap.data() + d->layout_index(1, y, z), 0, static_cast<size_t>(g.xl));
        d->ops->init(d->dev, d->stream);
        check(cudaGetLastError(), "init kernel");
        check(cudaStreamSynchronize(d->stream), "init");
    });
    if (rc != LBM_OK) {
        g_create_error = d->err;
        delete d;
        return rc;
    }
    *out = d;
    return LBM_OK;
}

void lbm_destroy(lbm_domain* d)
{
    if (!d) return;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev >= 0 && prev != d->device) cudaSetDevice(d->device);
    const int dev = d->device;
    if (d->stream) cudaStreamSynchronize(d->stream);
    delete d;  // frees the handle's memory on its device
    if (prev >= 0 && prev != dev) cudaSetDevice(prev);
}

int lbm_add_boundary(lbm_domain* d, int type, const double params[4], int* handler)
{
    return guarded(d, [&] {
        if (type < LBM_NOSLIP || type > LBM_PRESSURE) throw ArgError("unknown boundary type");
        if (static_cast<int>(d->bcs.size()) >= kMaxHandlers) throw ArgError("too many boundary handlers");
        BcEntry b{};
        b.type = type;
        b.has_profile = 0;
        if (params) {
            for (int k = 0; k < 4; ++k)
                if (!std::isfinite(params[k])) throw ArgError("boundary parameters must be finite");
            b.v[0] = params[0]; b.v[1] = params[1]; b.v[2] = params[2];
            b.rho = params[3];
        } else {
            b.rho = 1.0;
        }
        if ((type == LBM_OUTFLOW || type == LBM_PRESSURE) && b.rho == 0.0)
            throw ArgError("reference density must be nonzero");
        d->bcs.push_back(b);
        d->profiles.emplace_back();
        d->geom_dirty = true;
        if (handler) *handler = static_cast<int>(d->bcs.size());
    });
}

int lbm_set_boundary_box(lbm_domain* d, int handler, const int64_t box[6])
{
    return guarded(d, [&] {
        if (handler < 1 || handler > static_cast<int>(d->bcs.size())) throw ArgError("unknown handler");
        if (!box) throw ArgError("box is NULL");
        const Geom& g = d->dev.g;
        // domain.hpp:180-181
        if (!(box[1] >= box[0] && box[3] >= box[2] && box[5] >= box[4])) throw ArgError("box end before begin");
        if (box[0] < 0 || box[2] < 0 || box[4] < 0 || box[1] >= g.xl + 2 || box[3] >= g.yl + 2 || box[5] >= g.zl + 2)
            throw ArgError("box outside the domain (ghost layer included)");
        const uint8_t v = static_cast<uint8_t>(kFirstHandler + handler - 1);
        for (int64_t z = box[4]; z <= box[5]; ++z)
            for (int64_t y = box[2]; y <= box[3]; ++y)
                std::memset(d->hmap.data() + d->layout_index(static_cast<int>(box[0]), static_cast<int>(y), static_cast<int>(z)),
                            v, static_cast<size_t>(box[1] - box[0] + 1));
        d->geom_dirty = true;
    });
}

int lbm_set_solid_mask(lbm_domain* d, const uint8_t* mask, int* handler)
{
    return guarded(d, [&] {
        if (!mask) throw ArgError("mask is NULL");
        if (static_cast<int>(d->bcs.size()) >= kMaxHandlers) throw ArgError("too many boundary handlers");
        BcEntry b{};
        b.type = kNoSlip;
        b.rho = 1.0;
        d->bcs.push_back(b);
        d->profiles.emplace_back();
        const int h = static_cast<int>(d->bcs.size());
        const uint8_t v = static_cast<uint8_t>(kFirstHandler + h - 1);
        const Geom& g = d->dev.g;
        size_t m = 0;
        for (int z = 1; z <= g.zl; ++z)
            for (int y = 1; y <= g.yl; ++y) {
                uint8_t* row = d->hmap.data() + d->layout_index(1, y, z);
                for (int x = 0; x < g.xl; ++x, ++m)
                    if (mask[m]) row[x] = v;
            }
        d->geom_dirty = true;
        if (handler) *handler = h;
    });
}

int lbm_set_periodic(lbm_domain* d, int px, int py, int pz)
{
    return guarded(d, [&] {
        d->dev.g.per = (px ? 1 : 0) | (py ? 2 : 0) | (pz ? 4 : 0);
        d->geom_dirty = true;
    });
}

int lbm_set_inflow_profile(lbm_domain* d, int handler, const double* u_cells)
{
    return guarded(d, [&] {
        if (handler < 1 || handler > static_cast<int>(d->bcs.size())) throw ArgError("unknown handler");
        if (d->bcs[handler - 1].type != kInflow) throw ArgError("handler is not an inflow boundary");
        if (!u_cells) throw ArgError("u_cells is NULL");
        d->profiles[handler - 1].assign(u_cells, u_cells + 3 * d->ng);
        d->bcs[handler - 1].has_profile = 1;
        d->geom_dirty = true;
    });
}

int lbm_set_nonfluid_cells_nullcollide(lbm_domain* d)
{
    return guarded(d, [&] {});
}

int lbm_set_populations(lbm_domain* d, const double* f)
{
    return guarded(d, [&] {
        if (!f) throw ArgError("f is NULL");
        d->finalize();
        d->adj.ready = false;
        d->upload_state(f);
        d->state_custom = true;
    });
}

int lbm_get_populations(lbm_domain* d, double* f)
{
    return guarded(d, [&] {
        if (!f) throw ArgError("f is NULL");
        d->finalize();
        d->download_state(f);
        d->check_device_error();
    });
}

int lbm_step(lbm_domain* d, int64_t nsteps)
{
    return guarded(d, [&] {
        if (nsteps < 0) throw ArgError("nsteps must be >= 0");
        d->finalize();
        for (int64_t k = 0; k < nsteps; ++k) d->ops->step(d->dev, d->steps + 1 + k, -1, nullptr, nullptr, d->stream);
        if (nsteps > 0) d->adj.ready = false;
        check(cudaGetLastError(), "step kernel launch");
        d->steps += nsteps;
        if (nsteps > 0) d->state_custom = true;
    });
}

int lbm_step_monitored(lbm_domain* d, int64_t nsteps, double* totals)
{
    return guarded(d, [&] {
        if (nsteps < 0) throw ArgError("nsteps must be >= 0");
        if (!totals && nsteps > 0) throw ArgError("totals is NULL");
        d->finalize();
        // Step k adds into accumulator set k % 2; its totals land in ring slot k % kMonRing when the
        // next step's first block (or, after the last step, the fold kernel) adds that set up. The
        // ring goes to the host in whole groups of kMonRing slots, and the rest after the last fold.
        auto slot = [&](int64_t k) { return d->mon_ring.p + 4 * (k % kMonRing); };
        auto copy_out = [&](int64_t k0, int64_t n) {
            check(cudaMemcpyAsync(totals + 4 * k0, slot(k0), static_cast<size_t>(n) * 4 * sizeof(double),
                                  cudaMemcpyDeviceToHost, d->stream),
                  "copy step totals");
        };
        int64_t copied = 0;
        for (int64_t k = 0; k < nsteps; ++k) {
            d->ops->step(d->dev, d->steps + 1 + k, static_cast<int>(k & 1), k > 0 ? slot(k - 1) : nullptr, nullptr,
                         d->stream);
            if (k - copied == kMonRing) {  // slots copied .. k - 1 are written
                copy_out(copied, kMonRing);
                copied = k;
            }
        }
        if (nsteps > 0) {
            d->ops->monitor_fold(d->dev, static_cast<int>((nsteps - 1) & 1), slot(nsteps - 1), d->stream);
            copy_out(copied, nsteps - copied);
        }
        check(cudaGetLastError(), "step kernel launch");
        d->steps += nsteps;
        if (nsteps > 0) d->state_custom = true;
        if (nsteps > 0) d->adj.ready = false;
    });
}

int lbm_moments(lbm_domain* d, double* rho, double* u)
{
    return guarded(d, [&] {
        if (!rho) throw ArgError("rho is NULL");
        d->finalize();
        d->download_moments(rho, u);
        d->check_device_error();
    });
}

int lbm_moments_noalloc(lbm_domain* d, double* rho, double* u)
{
    return guarded(d, [&] {
        if (!rho) throw ArgError("rho is NULL");
        if (d->geom_dirty)
            throw StateError("the geometry changed since the last step; call lbm_step (or lbm_moments) once before "
                             "lbm_moments_noalloc, which never allocates and so cannot apply the change");
        if (d->n_interior > kNoAllocMaxCells)
            throw ArgError("lbm_moments_noalloc handles at most 262144 interior cells (its static device scratch); "
                           "this domain has " + std::to_string(d->n_interior) + ": use lbm_moments");
        int prev = -1;
        check(cudaGetDevice(&prev), "cudaGetDevice");
        if (prev != d->device) check(cudaSetDevice(d->device), "cudaSetDevice");
        struct Restore {
            int dev, prev;
            ~Restore() { if (prev >= 0 && prev != dev) cudaSetDevice(prev); }
        } restore{d->device, prev};
        double* scratch = noalloc_scratch(d->device);
        d->ops->moments(d->dev, d->steps, scratch, u ? scratch + d->n_interior : nullptr, d->stream);
        check(cudaGetLastError(), "moments kernel");
        check(cudaMemcpyAsync(rho, scratch, d->n_interior * sizeof(double), cudaMemcpyDeviceToHost, d->stream),
              "download density");
        if (u)
            check(cudaMemcpyAsync(u, scratch + d->n_interior, 3 * d->n_interior * sizeof(double),
                                  cudaMemcpyDeviceToHost, d->stream),
                  "download velocity");
        check(cudaStreamSynchronize(d->stream), "moments");
        d->check_device_error();
    });
}

int lbm_reduce_mass_momentum(lbm_domain* d, double out[4])
{
    bool diverged = false;
    const int rc = guarded(d, [&] {
        if (!out) throw ArgError("out is NULL");
        d->finalize();
        double* partials = d->red.p;
        double* total = d->red.p + 4 * kReduceBlocks;
        d->ops->reduce(d->dev, d->steps, partials, kReduceBlocks, total, d->stream);
        check(cudaGetLastError(), "reduction kernel");
        check(cudaMemcpyAsync(out, total, 4 * sizeof(double), cudaMemcpyDeviceToHost, d->stream), "download totals");
        check(cudaStreamSynchronize(d->stream), "reduction");
        d->check_device_error();
        for (int k = 0; k < 4; ++k) diverged = diverged || !std::isfinite(out[k]);
        if (diverged) d->err = "non-finite mass or momentum: the run diverged";
    });
    if (rc == LBM_OK && diverged) return LBM_ERR_DIVERGED;
    return rc;
}

int lbm_sync(lbm_domain* d)
{
    return guarded(d, [&] {
        check(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        d->check_device_error();
    });
}

int lbm_get_stream(lbm_domain* d, void** stream)
{
    return guarded(d, [&] {
        if (!stream) throw ArgError("stream is NULL");
        *stream = static_cast<void*>(d->stream);
    });
}

int64_t lbm_steps_done(const lbm_domain* d) { return d ? d->steps : -1; }

int lbm_memory_info(const lbm_domain* d, uint64_t* device_bytes, uint64_t* step_bytes, uint64_t* fluid_cells,
                    uint64_t* launches_per_step)
{
    if (!d) return LBM_ERR_ARG;
    lbm_domain* m = const_cast<lbm_domain*>(d);
    return guarded(m, [&] {
        m->finalize();
        if (device_bytes)
            *device_bytes = m->pop.bytes() + m->flag.bytes() + m->bc.bytes() + m->profile.bytes() + m->gf_xyz.bytes() +
                            m->gf_pop.bytes() + m->fs_link.bytes() + m->red.bytes() + m->link.bytes() + m->edge.bytes() +
                            m->errword.bytes() + m->mon.bytes() + m->mon_ring.bytes() + m->stage.bytes() + m->ltab.bytes() +
                            m->wmask.bytes() + m->adj.mu[0].bytes() + m->adj.mu[1].bytes() + m->adj.rec.bytes() + m->adj.rec2.bytes() + m->adj.backup.bytes() +
                            m->adj.gin.bytes() + m->adj.gwall.bytes();
        if (device_bytes)
            for (const auto& c : m->adj.ckpt) *device_bytes += c->bytes();
        if (step_bytes) *step_bytes = 2ull * m->Q * store_bytes(m->precision) * m->fluid_cells;
        if (fluid_cells) *fluid_cells = m->fluid_cells;
        if (launches_per_step)
            *launches_per_step = 1 + (m->dev.n_gf > 0) + (m->dev.n_fs > 0);
    });
}

namespace {

Box to_box(const lbm_domain* d, const int64_t box[6])
{
    if (!box) throw ArgError("box is NULL");
    const Geom& g = d->dev.g;
    if (!(box[0] >= 1 && box[0] <= box[1] && box[1] <= g.xl && box[2] >= 1 && box[2] <= box[3] &&
          box[3] <= g.yl && box[4] >= 1 && box[4] <= box[5] && box[5] <= g.zl))
        throw ArgError("objective box must be a non-empty box of interior cells");
    return Box{static_cast<int>(box[0]), static_cast<int>(box[1]), static_cast<int>(box[2]),
               static_cast<int>(box[3]), static_cast<int>(box[4]), static_cast<int>(box[5])};
}

}  // namespace

int lbm_adjoint_forward(lbm_domain* d, int64_t nsteps, int64_t ckpt_every)
{
    return guarded(d, [&] {
        if (nsteps < 1 || ckpt_every < 1) throw ArgError("nsteps and ckpt_every must be >= 1");
        d->finalize();
        if (d->dev.n_fs > 0 || d->dev.n_gf > 0)
            throw StateError("gradients are not available with free-slip cells or ghost cells without a handler");
        AdjointRun& a = d->adj;
        a.ready = false;
        a.ckpt.clear();
        a.s0 = d->steps;
        a.n = nsteps;
        a.k = ckpt_every;
        a.resident = ckpt_every == 1;
        // a record buffer of another size (a previous run's) goes before this run allocates
        const size_t rec_bytes = 4 * d->dev.g.PS * d->ops->compute_bytes;
        const size_t rec_need = static_cast<size_t>(a.resident ? nsteps : ckpt_every) * rec_bytes;
        if (a.rec.bytes() != rec_need) a.rec.release();
        if (a.resident) {
            // every step records its cell moments (what the backward's recompute would record)
            a.backup.release();
            a.rec2.release();
            if (!a.rec.p) a.rec.alloc(rec_need, "cudaMalloc(step records)");
            for (long long r = 0; r < nsteps; ++r)
                d->ops->step(d->dev, d->steps + 1 + r, -1, nullptr, a.rec.p + r * rec_bytes, d->stream);
            d->steps += nsteps;
            check(cudaGetLastError(), "step kernel launch");
            d->state_custom = true;
            a.ready = true;
            return;
        }
        const long long nseg = (nsteps + ckpt_every - 1) / ckpt_every;
        for (long long j = 0; j < nseg; ++j) {
            a.ckpt.emplace_back(new DevBuf<unsigned char>());
            a.ckpt.back()->alloc(d->pop.bytes(), "cudaMalloc(checkpoint)");
        }
        for (long long j = 0; j < nseg; ++j) {
            check(cudaMemcpyAsync(a.ckpt[j]->p, d->pop.p, d->pop.bytes(), cudaMemcpyDeviceToDevice, d->stream),
                  "store checkpoint");
            const long long len = std::min<long long>(ckpt_every, nsteps - j * ckpt_every);
            for (long long r = 0; r < len; ++r) d->ops->step(d->dev, d->steps + 1 + r, -1, nullptr, nullptr, d->stream);
            d->steps += len;
        }
        check(cudaGetLastError(), "step kernel launch");
        d->state_custom = true;
        a.ready = true;
    });
}

int lbm_adjoint_objective_ke(lbm_domain* d, const int64_t box[6], double* J)
{
    return guarded(d, [&] {
        if (!J) throw ArgError("J is NULL");
        d->finalize();
        const Box b = to_box(d, box);
        double* partials = d->red.p;
        double* total = d->red.p + 4 * kReduceBlocks;
        d->ops->objective_ke(d->dev, d->steps, b, partials, kReduceBlocks, total, d->stream);
        check(cudaGetLastError(), "objective kernel");
        check(cudaMemcpyAsync(J, total, sizeof(double), cudaMemcpyDeviceToHost, d->stream), "download objective");
        check(cudaStreamSynchronize(d->stream), "objective");
        d->check_device_error();
    });
}

int lbm_adjoint_backward(lbm_domain* d, const int64_t box[6], double dJ, double* grad_inflow, double* grad_wall)
{
    return guarded(d, [&] {
        AdjointRun& a = d->adj;
        if (!a.ready || d->steps != a.s0 + a.n || d->geom_dirty)
            throw StateError("lbm_adjoint_backward needs the state lbm_adjoint_forward left (no steps, "
                             "population writes or geometry changes in between)");
        const Box b = to_box(d, box);
        const size_t PS = d->dev.g.PS;
        const size_t Tb = d->ops->compute_bytes;
        const size_t rec_bytes = 4 * PS * Tb;
        auto& mu = a.mu;
        auto& rec = a.rec;
        auto& backup = a.backup;
        auto& gin = a.gin;
        auto& gwall = a.gwall;
        const size_t mu_bytes = static_cast<size_t>(d->Q) * PS * Tb;
        if (mu[0].bytes() != mu_bytes) {
            mu[0].alloc(mu_bytes, "cudaMalloc(adjoint populations)");
            mu[1].alloc(mu_bytes, "cudaMalloc(adjoint populations)");
            gin.alloc(3 * d->ng, "cudaMalloc(inflow gradient)");
            gwall.alloc(3 * kMaxHandlers, "cudaMalloc(wall gradient)");
        }
        const long long nseg = a.resident ? 1 : static_cast<long long>(a.ckpt.size());
        if (a.resident) {
            backup.release();  // no recompute: the state is never touched
        } else {
            const size_t seg_rec = static_cast<size_t>(a.k) * rec_bytes;
            if (rec.bytes() != seg_rec) rec.alloc(seg_rec, "cudaMalloc(recompute record)");
            if (nseg > 1 && a.rec2.bytes() != seg_rec) a.rec2.alloc(seg_rec, "cudaMalloc(recompute record)");
            if (backup.bytes() != d->pop.bytes()) backup.alloc(d->pop.bytes(), "cudaMalloc(state backup)");
            if (!a.rstream) {
                check(cudaStreamCreateWithFlags(&a.rstream, cudaStreamNonBlocking), "cudaStreamCreate(recompute)");
                for (int k = 0; k < 2; ++k) {
                    check(cudaEventCreateWithFlags(&a.filled[k], cudaEventDisableTiming), "cudaEventCreate");
                    check(cudaEventCreateWithFlags(&a.drained[k], cudaEventDisableTiming), "cudaEventCreate");
                }
            }
        }
        check(cudaMemsetAsync(gin.p, 0, gin.bytes(), d->stream), "clear gradient");
        check(cudaMemsetAsync(gwall.p, 0, gwall.bytes(), d->stream), "clear gradient");
        check(cudaMemsetAsync(mu[0].p, 0, mu[0].bytes(), d->stream), "clear adjoint");
        check(cudaMemsetAsync(mu[1].p, 0, mu[1].bytes(), d->stream), "clear adjoint");
        if (!a.resident)
            check(cudaMemcpyAsync(backup.p, d->pop.p, d->pop.bytes(), cudaMemcpyDeviceToDevice, d->stream),
                  "state backup");

        // resident: one segment of all n steps whose records the forward wrote. Otherwise segment
        // j is recomputed from its checkpoint on the recompute stream into record buffer j % 2
        // while the handle's stream runs the adjoint steps of segment j + 1 from the other buffer:
        // both kernels are latency-bound on small domains and fill the GPU together. The adjoint
        // steps touch no population; the recompute waits until its buffer has been read.
        const long long seg_len = a.resident ? a.n : a.k;
        unsigned char* const recs[2] = {rec.p, a.rec2.p};
        auto recompute = [&](long long j) {
            const int bj = static_cast<int>(j & 1);
            const long long c = a.s0 + j * seg_len;
            const long long len = std::min<long long>(seg_len, a.n - j * seg_len);
            check(cudaStreamWaitEvent(a.rstream, a.drained[bj], 0), "recompute wait");
            check(cudaMemcpyAsync(d->pop.p, a.ckpt[j]->p, d->pop.bytes(), cudaMemcpyDeviceToDevice, a.rstream),
                  "restore checkpoint");
            for (long long r = 1; r <= len; ++r)  // recording rec_{c+r}
                d->ops->step(d->dev, c + r, -1, nullptr, recs[bj] + (r - 1) * rec_bytes, a.rstream);
            check(cudaEventRecord(a.filled[bj], a.rstream), "recompute done");
        };
        if (!a.resident) {
            // both buffers free, after the clears and the state backup above
            for (int k = 0; k < 2; ++k) check(cudaEventRecord(a.drained[k], d->stream), "adjoint start");
            recompute(nseg - 1);
        }
        int cur = 0;
        long long t_cur = 0;  // mu[cur] holds mu_{t_cur}
        for (long long j = nseg - 1; j >= 0; --j) {
            const int bj = static_cast<int>(j & 1);
            const long long c = a.s0 + j * seg_len;
            const long long len = std::min<long long>(seg_len, a.n - j * seg_len);
            const unsigned char* rj = a.resident ? rec.p : recs[bj];
            if (!a.resident) {
                if (j > 0) recompute(j - 1);  // runs alongside this segment's adjoint steps
                check(cudaStreamWaitEvent(d->stream, a.filled[bj], 0), "adjoint wait");
            }
            if (j == nseg - 1) {
                d->ops->adj_terminal(d->dev, rj + (len - 1) * rec_bytes, mu[cur].p, b, d->stream);
                t_cur = c + len;
            }
            // mu_t -> mu_{t-1} with the record of step t-1; the run's first step (t = s0 + 1) pulls
            // the boundary values the starting state holds, so the loop ends at t = s0 + 2
            for (long long t = t_cur; t >= c + 2; --t) {
                d->ops->adj_step(d->dev, mu[cur].p, mu[1 - cur].p, rj + (t - c - 2) * rec_bytes, 1, 1, gin.p,
                                 gwall.p, d->stream);
                cur = 1 - cur;
                t_cur = t - 1;
            }
            if (!a.resident) check(cudaEventRecord(a.drained[bj], d->stream), "adjoint segment done");
        }
        if (!a.resident)
            check(cudaMemcpyAsync(d->pop.p, backup.p, d->pop.bytes(), cudaMemcpyDeviceToDevice, d->stream),
                  "restore state");
        // times the upstream gradient on the device, then straight into the caller's arrays
        scale_doubles(gin.p, gin.n, dJ, d->stream);
        scale_doubles(gwall.p, gwall.n, dJ, d->stream);
        check(cudaGetLastError(), "adjoint kernels");
        if (grad_inflow) {
            check(cudaMemcpyAsync(grad_inflow, gin.p, gin.bytes(), cudaMemcpyDeviceToHost, d->stream),
                  "download inflow gradient");
        }
        if (grad_wall && !d->bcs.empty())
            check(cudaMemcpyAsync(grad_wall, gwall.p, 3 * d->bcs.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  d->stream),
                  "download wall gradient");
        check(cudaStreamSynchronize(d->stream), "adjoint");
        d->check_device_error();
    });
}

const char* lbm_last_error(const lbm_domain* d)
{
    if (!d) return g_create_error.c_str();
    return d->err.c_str();
}

}  // extern "C"
