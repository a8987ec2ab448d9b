// imexlbm: drop-in driver for the reference's single-rank main loop
// (src/main.cpp:6-110).  Reads ./input.in (or the path given as the first
// argument), prints the same banner, "rx=..." line, per-step "collision"
// lines (unless --no-perstep-timing, the reference's LBM_NO_PERSTEP_TIMING
// build), "step ... MLUPS" lines and "cons  step ..." lines with the same
// printf formats, so tests/regression.sh-style parsers read it unchanged.
//
// Timing note: Collision() launches the fused stream+collide kernel and
// Streaming() only marks the streaming as pending, so the per-step
// "collision" line times the whole step.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>

#include "lbm.hpp"

static double wtime()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char* argv[])
{
    bool perstep = true;
    const char* deck = "input.in";
    int precision = IMEX_F64;
    int engine = IMEX_ENGINE_AUTO;
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
        else if (argv[i][0] != '-')
            deck = argv[i];
        else {
            std::fprintf(stderr,
                         "usage: imexlbm [deck] [--no-perstep-timing] [--engine=native|fixed] "
                         "[--precision=f64|f32|f16dev]\n");
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
        l1.fence();
        const double start = wtime();
        double t_last = start;
        for (int it = 1; it <= s1.Time; it++) {
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
            }
            l1.Streaming();
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
                t_last = wtime();
            }
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
