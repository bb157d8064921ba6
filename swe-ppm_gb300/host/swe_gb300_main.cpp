// swe_gb300 -- the drivers' checkpoint loop on the GB300 block step.
//
// Same flags and output as the reference drivers (src/examples/swe_mpi.cpp:70-82,
// swe_mpi_overdecomp.cpp): -t simulated seconds, -n checkpoints, -x/-y cells,
// -o output base name, -w 1 to write NetCDF files (one per block, like one per
// rank), plus --blocks N (overdecomposition into a near-square block grid),
// --solver hlle|fwave|augrie|hybrid, --semantics unsplit|split, --scenario,
// --seed and --arithmetic exact|fast (the fast-arithmetic step of the f-wave
// and HLLE solvers).  The time loop `while (t < checkpoint) step` of
// src/examples/swe_mpi.cpp:300-327 runs on the device (swe_gpu_advance, or
// swe_gpu_lts_advance with -l > 0: local time stepping with intervals of that
// length, src/examples/swe_mpi_overdecomp.cpp:308-343); at
// every checkpoint each block's state is snapshotted asynchronously into
// pinned buffers and a writer thread appends it to the block's NetCDF file
// while the next interval runs.  A Collector-style CSV line (PE_COUNT,
// FLOP_COUNT, FLOPS, WALL_TIME, COMMUNICATION_TIME, REDUCTION_TIME;
// src/tools/Collector.hpp:116-144) with the reference's 135-flop-per-edge
// model is appended to <output>.log.
#include <getopt.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/swe_gb300.h"
#include "../../include/swe_gb300_host.h"

namespace {

void die(const char *what) {
    fprintf(stderr, "swe_gb300: %s: %s\n", what, swe_gpu_last_error());
    exit(1);
}

int scenarioId(const std::string &s) {
    if (s == "radial_bathymetry_dam_break") return SWE_SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK;
    if (s == "radial_dam_break") return SWE_SCENARIO_RADIAL_DAM_BREAK;
    if (s == "half_domain_dry") return SWE_SCENARIO_HALF_DOMAIN_DRY;
    if (s == "sea_at_rest") return SWE_SCENARIO_SEA_AT_REST;
    if (s == "dam_break") return SWE_SCENARIO_DAM_BREAK;
    if (s == "tsunami") return SWE_SCENARIO_TSUNAMI;
    if (s == "shoreline") return SWE_SCENARIO_SHORELINE;
    return -1;
}

int solverId(const std::string &s) {
    if (s == "fwave") return SWE_SOLVER_FWAVE;
    if (s == "augrie") return SWE_SOLVER_AUGRIE;
    if (s == "hybrid") return SWE_SOLVER_HYBRID;
    return SWE_SOLVER_HLLE;
}

/// one checkpoint's snapshot of every block, written by the writer thread
struct Slot {
    std::vector<void *> bufs;  // 3 pinned slabs per block
    float t = 0.f;
    bool full = false;
};

} // namespace

int main(int argc, char **argv) {
    float duration = 0.f;
    int checkpoints = 1, nx = 0, ny = 0, nblocks = 1, write = 0, semantics = SWE_SEMANTICS_UNSPLIT;
    int arithmetic = SWE_ARITH_EXACT;
    float ltsInterval = 0.f;  // -l: local time stepping with intervals of this length
    std::string out = "swe", scenario = "radial_bathymetry_dam_break", solver = "hlle";
    double seed = 20261203;
    static option opts[] = {{"simulation-duration", required_argument, 0, 't'},
                            {"checkpoint-count", required_argument, 0, 'n'},
                            {"resolution-horizontal", required_argument, 0, 'x'},
                            {"resolution-vertical", required_argument, 0, 'y'},
                            {"output-basepath", required_argument, 0, 'o'},
                            {"write", required_argument, 0, 'w'},
                            {"local-timestepping", required_argument, 0, 'l'},
                            {"blocks", required_argument, 0, 'b'},
                            {"solver", required_argument, 0, 's'},
                            {"semantics", required_argument, 0, 'm'},
                            {"scenario", required_argument, 0, 'c'},
                            {"seed", required_argument, 0, 'e'},
                            {"arithmetic", required_argument, 0, 'a'},
                            {0, 0, 0, 0}};
    int c;
    while ((c = getopt_long(argc, argv, "t:n:x:y:o:w:l:b:s:m:c:e:a:", opts, nullptr)) != -1) {
        switch (c) {
        case 't': duration = float(atof(optarg)); break;
        case 'n': checkpoints = atoi(optarg); break;
        case 'x': nx = atoi(optarg); break;
        case 'y': ny = atoi(optarg); break;
        case 'o': out = optarg; break;
        case 'w': write = atoi(optarg); break;
        case 'l': ltsInterval = float(atof(optarg)); break;
        case 'b': nblocks = atoi(optarg); break;
        case 's': solver = optarg; break;
        case 'm': semantics = std::string(optarg) == "split" ? SWE_SEMANTICS_SPLIT : SWE_SEMANTICS_UNSPLIT; break;
        case 'c': scenario = optarg; break;
        case 'e': seed = atof(optarg); break;
        case 'a': arithmetic = std::string(optarg) == "fast" ? SWE_ARITH_FAST : SWE_ARITH_EXACT; break;
        default:
            fprintf(stderr, "usage: %s -t seconds -n checkpoints -x nx -y ny [-o base] [-w 1] [--blocks N] "
                            "[--solver hlle|fwave|augrie|hybrid] [--semantics unsplit|split] [--scenario name] "
                            "[--arithmetic exact|fast]\n",
                    argv[0]);
            return 1;
        }
    }
    const int sid = scenarioId(scenario);
    if (sid < 0 || nx < 1 || ny < 1 || checkpoints < 1) {
        fprintf(stderr, "swe_gb300: need -t, -n, -x, -y and a known --scenario\n");
        return 1;
    }
    double params[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (sid == SWE_SCENARIO_TSUNAMI) {
        params[0] = nx;
        params[1] = seed;
    } else if (sid == SWE_SCENARIO_SHORELINE) {
        params[0] = seed;
    }

    // checkpoint instants, accumulated in float (src/examples/swe_mpi.cpp:132-139)
    std::vector<float> cp(checkpoints);
    const float delta = duration / checkpoints;
    cp[0] = delta;
    for (int i = 1; i < checkpoints; i++) cp[i] = cp[i - 1] + delta;

    float geo[4];
    int outer[4];
    if (swe_host_scenario_geometry(sid, params, nx, ny, geo) || swe_host_scenario_boundary(sid, params, outer))
        die("scenario");
    int bx = 0, by = 0;
    std::vector<int> cols(nblocks), rows(nblocks);
    std::vector<float> ox(nblocks), oy(nblocks);
    if (swe_host_decompose(nx, ny, nblocks, geo[0], geo[1], geo[2], geo[3], &bx, &by, cols.data(), rows.data(),
                           ox.data(), oy.data()))
        die("decomposition");

    swe_gpu_desc d{};
    d.blocks_x = bx;
    d.blocks_y = by;
    d.nx_cols = cols.data();
    d.ny_rows = rows.data();
    d.dx = geo[0];
    d.dy = geo[1];
    for (int i = 0; i < 4; i++) d.boundary[i] = outer[i];
    d.solver = solverId(solver);
    d.semantics = semantics;
    d.lts_max_timestep = ltsInterval;
    d.duration = duration;
    d.arithmetic = arithmetic;
    swe_gpu_domain *dom = nullptr;
    if (swe_gpu_domain_create(&d, &dom)) die("swe_gpu_domain_create");

    // initScenario of every block (neighbour sides connect within the domain)
    std::vector<std::vector<float>> bathy(bx * by);
    for (int k = 0; k < bx * by; k++) {
        const int px = k / by, py = k % by;
        const int bnd[4] = {px > 0 ? SWE_CONNECT_WITHIN_RANK : outer[0], px < bx - 1 ? SWE_CONNECT_WITHIN_RANK : outer[1],
                            py > 0 ? SWE_CONNECT_WITHIN_RANK : outer[2], py < by - 1 ? SWE_CONNECT_WITHIN_RANK : outer[3]};
        const size_t n = size_t(cols[px] + 2) * size_t(rows[py] + 2);
        std::vector<float> h(n), hu(n), hv(n);
        bathy[k].resize(n);
        if (swe_host_init_block(sid, params, cols[px], rows[py], geo[0], geo[1], ox[px], oy[py], bnd, h.data(),
                                hu.data(), hv.data(), bathy[k].data(), rows[py] + 2))
            die("init");
        if (swe_gpu_upload_block(dom, k, h.data(), hu.data(), hv.data(), bathy[k].data(), rows[py] + 2)) die("upload");
    }
    if (swe_gpu_exchange_bathymetry(dom)) die("exchange bathymetry");
    for (int k = 0; k < bx * by; k++) {  // b with its neighbour ghosts, for the writers
        const int py = k % by;
        if (swe_gpu_download_block(dom, k, nullptr, nullptr, nullptr, bathy[k].data(), rows[py] + 2)) die("download");
    }

    // writers: one NetCDF file per block, fed by a thread from two pinned slots
    std::vector<swe_nc_writer *> writers(bx * by, nullptr);
    Slot slots[2];
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    std::thread writerThread;
    if (write) {
        for (int k = 0; k < bx * by; k++) {
            const int px = k / by, py = k % by;
            const std::string path = out + "_" + std::to_string(k) + ".nc";
            if (swe_nc_open(path.c_str(), cols[px], rows[py], geo[0], geo[1], ox[px], oy[py], bathy[k].data(),
                            rows[py] + 2, &writers[k]))
                die(("open " + path).c_str());
            std::vector<float> h(bathy[k].size()), hu(h.size()), hv(h.size());
            if (swe_gpu_download_block(dom, k, h.data(), hu.data(), hv.data(), nullptr, rows[py] + 2)) die("download");
            swe_nc_write_step(writers[k], 0.f, h.data(), hu.data(), hv.data(), rows[py] + 2);  // t = 0
        }
        for (auto &s : slots)
            for (int k = 0; k < bx * by; k++) {
                const size_t bytes = size_t(cols[k / by]) * size_t(rows[k % by]) * 4;
                for (int f = 0; f < 3; f++) {
                    void *p = nullptr;
                    if (swe_gpu_alloc_pinned(bytes, &p)) die("pinned buffer");
                    s.bufs.push_back(p);
                }
            }
        writerThread = std::thread([&] {
            int next = 0;
            for (;;) {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return slots[next].full || stop; });
                if (!slots[next].full && stop) return;
                lk.unlock();
                for (int k = 0; k < bx * by; k++)
                    swe_nc_write_step_slabs(writers[k], slots[next].t, slots[next].bufs[3 * k],
                                            slots[next].bufs[3 * k + 1], slots[next].bufs[3 * k + 2]);
                lk.lock();
                slots[next].full = false;
                cv.notify_all();
                next ^= 1;
            }
        });
    }

    const auto t0 = std::chrono::steady_clock::now();
    long long steps = 0;
    float t = 0.f;
    for (int i = 0; i < checkpoints; i++) {
        int n = 0;
        if (ltsInterval > 0.f) {
            // the drivers' `while (t < checkpoint)` over synchronisation intervals
            if (swe_gpu_lts_advance(dom, cp[i], 1 << 30, &n, &t)) die("local time stepping");
        } else {
            if (swe_gpu_advance(dom, cp[i], 1 << 30, &n, &t)) die("advance");
            steps += n;
        }
        printf("Write timestep (%fs)\n", t);
        if (write) {
            Slot &s = slots[i & 1];
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return !s.full; });
            }
            for (int k = 0; k < bx * by; k++)
                if (swe_gpu_snapshot_slabs_async(dom, k, s.bufs[3 * k], s.bufs[3 * k + 1], s.bufs[3 * k + 2]) ||
                    swe_gpu_snapshot_wait(dom))
                    die("snapshot");
            std::lock_guard<std::mutex> lk(mu);
            s.t = t;
            s.full = true;
            cv.notify_all();
        }
    }
    if (swe_gpu_sync(dom)) die("sync");
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (write) {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
            cv.notify_all();
        }
        writerThread.join();
        for (auto *w : writers) swe_nc_close(w);
        for (auto &s : slots)
            for (void *p : s.bufs) swe_gpu_free_pinned(p);
    }
    // cell updates summed over blocks (under local time stepping blocks step
    // at their own rates)
    std::vector<long long> blockSteps(size_t(bx) * by);
    if (swe_gpu_block_steps(dom, blockSteps.data())) die("block steps");
    double cellUpdates = 0.0;
    steps = 0;
    for (int k = 0; k < bx * by; k++) {
        cellUpdates += double(cols[k / by]) * double(rows[k % by]) * double(blockSteps[k]);
        steps = std::max(steps, blockSteps[k]);
    }
    const double flops = 2.0 * 135.0 * cellUpdates;
    printf("Flop count: %g\nFlops: %gGFLOPS\nWall Time: %gs\nSteps: %lld\nCell updates: %g/s\n", flops,
           1e-9 * flops / wall, wall, steps, cellUpdates / wall);
    const std::string logName = out + ".log";
    const bool exists = std::ifstream(logName).good();
    std::ofstream log(logName, std::ios::app);
    if (!exists) log << "PE_COUNT,FLOP_COUNT,FLOPS,WALL_TIME,COMMUNICATION_TIME,REDUCTION_TIME\n";
    log << bx * by << "," << flops << "," << flops / wall << "," << wall << ",0,0\n";
    swe_gpu_domain_destroy(dom);
    return 0;
}
