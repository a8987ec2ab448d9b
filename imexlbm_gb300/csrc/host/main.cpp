// imexlbm: drop-in driver for the reference's single-rank main loop
// (src/main.cpp:6-110).  Reads ./input.in (or the path given as the first
// argument), prints the same banner, "rx=..." line, per-step "collision"
// lines (unless --no-perstep-timing, the reference's LBM_NO_PERSTEP_TIMING
// build), "step ... MLUPS" lines and "cons  step ..." lines with the same
// printf formats, so tests/regression.sh-style parsers read it unchanged.
//
// --profile prints the per-phase report of the reference's profiling build
// (src/profile.cpp:107-200, same table and group summary formats) at the
// end: STEP TOTAL is host wall time around Collision + Streaming, as there;
// the kernel rows are device times from CUDA events, so no fence is added.
// Step 1 is discarded as warm-up, as the reference does.
//
// --output writes output<it/inter>.plt at every report step, the call the
// reference leaves commented out at src/main.cpp:99 (off by default, as
// there).
//
// Timing note: Collision() launches the fused stream+collide kernel and
// Streaming() only marks the streaming as pending, so the per-step
// "collision" line times the whole step.  With --no-perstep-timing and no
// --profile nothing is printed between report steps, so the steps up to
// each report run as one LBM::Step call (imex_step: on the float64 engine a
// fixed-point run, the same numbers 8% faster at 256^3).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>

#include "lbm.hpp"

static double wtime()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Host-timed phase (calls, sum, fastest, slowest), as lbmprof keeps them.
struct HostPhase {
    double acc = 0, lo = 0, hi = 0, mark = 0;
    long calls = 0;
    void begin() { mark = wtime(); }
    void end()
    {
        const double dt = wtime() - mark;
        acc += dt;
        if (calls == 0 || dt < lo) lo = dt;
        if (calls == 0 || dt > hi) hi = dt;
        ++calls;
    }
};

// The per-phase report of src/profile.cpp:107-200 for one rank.  Device
// rows come from the lattice's phase statistics; bytes and flops per cell
// are the reference's (594 flops per collision, 189 per moments
// evaluation), bytes at the lattice's storage precision.
static void profile_report(const HostPhase& step, const imex_phase_stats* dev, int nsteps, long cells, int elem)
{
    if (nsteps <= 0) {
        std::printf("\n[profile] nothing to report (nsteps <= 0)\n");
        return;
    }
    // HBM copy bandwidth of the GPU for the "% BW" column: a GB300 measured
    // 6695.8 GB/s on a STREAM-style copy; IMEXLBM_PEAK_GBPS overrides it.
    double peak = 6695.8;
    if (const char* e = std::getenv("IMEXLBM_PEAK_GBPS")) peak = std::atof(e);
    struct Row {
        const char* name;
        long calls;
        double mean, lo, hi;
    };
    auto dev_row = [&](const char* name, int q) {
        const imex_phase_stats& d = dev[q];
        return Row{name, (long)d.calls, d.calls ? d.total_ms / d.calls : 0.0, d.min_ms, d.max_ms};
    };
    const Row stepr{"STEP TOTAL", step.calls, step.calls ? 1e3 * step.acc / step.calls : 0.0, 1e3 * step.lo,
                    1e3 * step.hi};
    const Row rows[4] = {dev_row("  collision (kernel)", IMEX_PHASE_COLLISION),
                         dev_row("  stream: kernel (alone)", IMEX_PHASE_STREAM),
                         dev_row("  computeMacroscopic", IMEX_PHASE_MACRO),
                         dev_row("  conserved (kernel)", IMEX_PHASE_CONSERVED)};
    std::printf("\n=== per-phase profile: %d ranks, %d timed steps ===\n", 1, nsteps);
    std::printf("mean ms = across-rank mean of each rank's per-step mean\n");
    std::printf("spread%% = (slowest step - fastest step) / mean, over all steps and\n");
    std::printf("          ranks. >20%% => the mean is not a stable number.\n");
    std::printf("imbal   = max/min ACROSS RANKS. >>1 means load imbalance.\n\n");
    std::printf("%-36s %9s %8s %8s %7s %6s %7s\n", "phase", "mean ms", "min ms", "max ms", "spread%", "imbal",
                "% step");
    std::printf("%-36s %9s %8s %8s %7s %6s %7s\n", "------------------------------------", "---------", "--------",
                "--------", "-------", "------", "-------");
    const double st = stepr.mean;
    auto line = [&](const Row& r) {
        std::printf("%-36s %9.4f %8.4f %8.4f %7.1f %6.2f %7.1f\n", r.name, r.mean, r.lo, r.hi,
                    r.mean > 0.0 ? 100.0 * (r.hi - r.lo) / r.mean : 0.0, r.mean > 0.0 ? 1.0 : 0.0,
                    st > 0.0 ? 100.0 * r.mean / st : 0.0);
    };
    line(stepr);
    double attributed = 0.0;
    for (const Row& r : rows)
        if (r.calls) {
            line(r);
            attributed += r.mean * r.calls / nsteps;  // per-step share of a phase not run every step
        }
    std::printf("%-36s %9.4f %8s %8s %7s %6s %7.1f\n", "  (unattributed)", st - attributed, "", "", "", "",
                st > 0.0 ? 100.0 * (st - attributed) / st : 0.0);

    std::printf("\n%-22s %9s %7s %10s %10s %7s\n", "group", "mean ms", "% step", "GFLOP/s", "GB/s", "% BW");
    std::printf("%-22s %9s %7s %10s %10s %7s\n", "----------------------", "---------", "-------", "----------",
                "----------", "-------");
    const double fb = (double)cells * 27 * elem;
    struct Group {
        const char* name;
        const Row& r;
        double bytes, flops;
    };
    const Group groups[4] = {{"collision", rows[0], 2.0 * fb, 594.0 * cells},
                             {"stream (enq+fence)", rows[1], 2.0 * fb, 0.0},
                             {"computeMacroscopic", rows[2], fb + 4.0 * cells * sizeof(double), 189.0 * cells},
                             {"conserved", rows[3], fb, 189.0 * cells}};
    for (const Group& g : groups) {
        if (!g.r.calls) continue;
        const double secs = g.r.mean * 1e-3;
        char gf[16], gb[16], bw[16];
        if (g.flops > 0.0 && secs > 0.0) std::snprintf(gf, sizeof gf, "%10.1f", g.flops / secs / 1e9);
        else std::snprintf(gf, sizeof gf, "%10s", "-");
        if (secs > 0.0) {
            const double gbps = g.bytes / secs / 1e9;
            std::snprintf(gb, sizeof gb, "%10.1f", gbps);
            std::snprintf(bw, sizeof bw, "%7.1f", 100.0 * gbps / peak);
        } else {
            std::snprintf(gb, sizeof gb, "%10s", "-");
            std::snprintf(bw, sizeof bw, "%7s", "-");
        }
        std::printf("%-22s %9.4f %7.1f %s %s %s\n", g.name, g.r.mean, st > 0.0 ? 100.0 * g.r.mean / st : 0.0, gf, gb,
                    bw);
    }
    std::printf("\nworkload/rank: %ld interior cells, halo %.2f MB send + %.2f MB recv\n", cells, 0.0, 0.0);
    std::printf("kernel rows are device times (CUDA events, no added fences); STEP TOTAL is host\n");
    std::printf("  wall time around Collision + Streaming.  Take throughput from the step lines.\n\n");
}

int main(int argc, char* argv[])
{
    bool perstep = true;
    const char* deck = "input.in";
    int precision = IMEX_F64;
    int engine = IMEX_ENGINE_AUTO;
    bool output = false;
    bool profile = false;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--no-perstep-timing"))
            perstep = false;
        else if (!std::strcmp(argv[i], "--engine=native"))
            engine = IMEX_ENGINE_NATIVE;
        else if (!std::strcmp(argv[i], "--engine=fixed"))
            engine = IMEX_ENGINE_FIXED;
        else if (!std::strcmp(argv[i], "--precision=f64"))
            precision = IMEX_F64;
        else if (!std::strcmp(argv[i], "--precision=f32"))
            precision = IMEX_F32;
        else if (!std::strcmp(argv[i], "--precision=f16dev"))
            precision = IMEX_F16DEV;
        else if (!std::strcmp(argv[i], "--output"))
            output = true;
        else if (!std::strcmp(argv[i], "--profile"))
            profile = true;
        else if (argv[i][0] != '-')
            deck = argv[i];
        else {
            std::fprintf(stderr,
                         "usage: imexlbm [deck] [--no-perstep-timing] [--engine=native|fixed] "
                         "[--precision=f64|f32|f16dev] [--output] [--profile]\n");
            return 2;
        }
    }
    try {
        System s1(deck);
        s1.Monitor();
        LBM l1(s1.sx, s1.sy, s1.sz, s1.tau, s1.rho0, s1.u0, precision);
        if (engine != IMEX_ENGINE_AUTO && imex_set_engine(l1.handle(), engine) != IMEX_OK)
            throw imex::Error(IMEX_ERR_ARG, imex_last_error(l1.handle()));
        std::printf("rx=%d,ry=%d,rz=%d\n", 1, 1, 1);  // setup_Cartesian on one rank
        l1.Initialize();
        // choose the fused step's launch shape now (the autotuner times the
        // candidates on this lattice) rather than inside the first timed steps
        int shape[4];
        if (imex_get_launch(l1.handle(), shape) != IMEX_OK) throw imex::Error(IMEX_ERR_CUDA, imex_last_error(l1.handle()));
        l1.fence();
        if (profile) l1.profile_enable(true);
        HostPhase p_step;
        imex_phase_stats dev[IMEX_NPHASE];
        const double start = wtime();
        double t_last = start;
        for (int it = 1; it <= s1.Time; it++) {
            if (!perstep && !profile) {
                // Nothing is reported between report steps: run the steps up to
                // the next one (or the end) in one call, which gives the same
                // numbers as a Collision()/Streaming() pair per step.
                int last = (it + s1.inter - 1) / s1.inter * s1.inter;
                if (last > s1.Time) last = s1.Time;
                l1.Step(last - it + 1);
                it = last;
            } else {
                if (profile) p_step.begin();
                if (perstep) {
                    l1.fence();
                    const double t0 = wtime();
                    l1.Collision();
                    l1.fence();
                    const double t1 = wtime();
                    const double collision_time = t1 - t0;
                    if (l1.me == 0) {
                        const double flop_per_cell = 594.0;
                        const double total_flop = flop_per_cell * s1.sx * s1.sy * s1.sz;
                        const double gflops = total_flop / collision_time / 1.0e9;
                        std::printf("collision | %8.4f ms | %10.2f GFLOPS\n", collision_time * 1e3, gflops);
                    }
                } else {
                    l1.Collision();
                    if (profile) l1.fence();  // the one fence the reference's profiling build adds
                }
                l1.Streaming();
                if (profile) {
                    p_step.end();
                    if (it == 1) {  // discard step 1 (first launch, autotuning)
                        p_step = HostPhase();
                        l1.profile_read(dev, true);
                    }
                }
            }
            if (it % s1.inter == 0) {
                l1.fence();
                const double now = wtime();
                if (l1.me == 0) {
                    const double dt_int = now - t_last;
                    const double mlups = (double)s1.sx * s1.sy * s1.sz * s1.inter / dt_int / 1.0e6;
                    std::printf("step %6d | interval %8.4f s | total %8.4f s | %10.2f MLUPS\n", it, dt_int,
                                now - start, mlups);
                }
                double mass, px, py, pz, ke;
                l1.Conserved(mass, px, py, pz, ke);
                if (l1.me == 0)
                    std::printf("cons  step %6d | mass %.15e | px %.15e | py %.15e | pz %.15e | ke %.15e\n", it,
                                mass, px, py, pz, ke);
                std::fflush(stdout);
                if (output) l1.MPIoutput(it / s1.inter);
                t_last = wtime();
            }
        }
        if (profile) {
            l1.profile_read(dev, false);
            profile_report(p_step, dev, s1.Time - 1, (long)s1.sx * s1.sy * s1.sz,
                           precision == IMEX_F64 ? 8 : precision == IMEX_F32 ? 4 : 2);
        }
    } catch (const imex::Error& e) {
        std::fprintf(stderr, "imexlbm: %s\n", e.what());
        return 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "imexlbm: %s\n", e.what());
        return 1;
    }
    return 0;
}
