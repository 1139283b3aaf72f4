// lbm_gb300_run: the reference's simulation driver (src/main.cpp:25-74) on lbm_gb300.
//
//   lbm_gb300_run config.cfg [--tau 0.6] [--timesteps N] ... [--model 15|19|27]
//                 [--precision fp64|fp32|fp16|bf16]
//
// Reads the configuration and the XML scenario it names, runs the time loop
// (stream/swap/collide), writes <output-dir>/<scenario name>.<t>.vts every timesteps-per-plot
// steps and prints MLUPS counted as the reference does ((xl+2)(yl+2)(zl+2) cells per step) and
// over the interior cells. The files are written on a background thread (lbm::io::VtkWriter)
// while the loop goes on; only the read-back of the moments is counted in the loop's time, as
// the reference counts none of its output. --model (the reference picks the lattice with -DD3Q=
// at compile time, main.cpp:3-13) and --precision are extensions.
#include <chrono>
#include <cstring>
#include <iostream>
#include <string>

#include "lbm_gb300_io.hpp"

namespace {

template <typename model>
int run(int argc, char** argv, int precision)
{
    lbm::io::Config cfg(argc, argv);
    auto collision = lbm::BGKCollision<model>(cfg.tau());
    auto domain = lbm::io::parse_scenario_file<model>(cfg.scenario_xml(), cfg, collision, precision);
    std::cout << cfg << std::endl;
    std::cout << "> Domain lengths (x,y,z): " << domain->xlength() << ", " << domain->ylength() << ", "
              << domain->zlength() << std::endl;
    std::cout << "Starting simulation..." << std::endl;
    domain->set_nonfluid_cells_nullcollide();
    lbm::io::VtkWriter writer;
    double seconds = 0.0;
    const auto wall0 = std::chrono::steady_clock::now();
    for (uint64_t t = 1; t <= cfg.timesteps(); ++t) {
        const auto t0 = std::chrono::steady_clock::now();
        domain->stream();
        domain->swap();
        domain->collide();
        if (cfg.timesteps_per_plot() && t % cfg.timesteps_per_plot() == 0) {
            lbm_sync(domain->native());
            seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            writer.submit(*domain, cfg.output_dir(), cfg.output_filename(), t);
        } else {
            seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    }
    const auto s0 = std::chrono::steady_clock::now();
    lbm_sync(domain->native());
    seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
    writer.finish();
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    const double xl = domain->xlength(), yl = domain->ylength(), zl = domain->zlength();
    std::cout << "Finished!" << std::endl;
    std::cout << "Total runtime: " << wall << " seconds." << std::endl;
    std::cout << "MLUPS: " << (2 + xl) * (2 + yl) * (2 + zl) * cfg.timesteps() / (seconds * 1e6) << std::endl;
    std::cout << "MLUPS (interior cells): " << xl * yl * zl * cfg.timesteps() / (seconds * 1e6) << std::endl;
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        int q = 19, precision = LBM_FP64;
        for (int i = 1; i + 1 < argc; ++i) {
            if (!std::strcmp(argv[i], "--model")) q = std::stoi(argv[i + 1]);
            if (!std::strcmp(argv[i], "--precision")) {
                const std::string p = argv[i + 1];
                precision = p == "fp32" ? LBM_FP32 : p == "fp16" ? LBM_FP16 : p == "bf16" ? LBM_BF16 : LBM_FP64;
            }
        }
        if (q == 15) return run<lbm::model::d3q15>(argc, argv, precision);
        if (q == 27) return run<lbm::model::d3q27>(argc, argv, precision);
        return run<lbm::model::d3q19>(argc, argv, precision);
    } catch (const std::exception& ex) {
        std::cerr << "An error occured: " << ex.what() << std::endl;
        return EXIT_FAILURE;
    }
}
