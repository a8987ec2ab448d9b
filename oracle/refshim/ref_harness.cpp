// Driver of the reference's own code, built from its unmodified src/ with
// the Kokkos / MPI stand-ins of this directory (test infrastructure).
//
//   imexref [--ranks N] [--threads T] main
//       run the reference's main() (src/main.cpp, compiled with its main
//       renamed imexref_main) on N ranks: it reads ./input.in and prints the
//       reference's own output lines
//   imexref [--ranks N] [--threads T] dump STEPS FILE [--tecplot K] [--ascii K]
//       System + LBM as src/main.cpp builds them, Initialize, STEPS times
//       Collision + Streaming with a "cons" line at every report step, then
//       the interior f of the whole lattice into FILE (float64, the
//       reference's order f[a][x][y][z]); optionally MPIoutput(K) and
//       Output(K) after ComputeMacroscopic
//
// Ranks are threads of this process (one thread per rank, T OpenMP
// threads inside each); MPI_Comm_rank answers each thread's own rank.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "shim_runtime.h"

#include "System.hpp"
#include "lbm.hpp"

int imexref_main(int argc, char* argv[]);

namespace {

std::vector<double> g_field;  // whole-lattice f of dump mode
int g_gx = 0, g_gy = 0, g_gz = 0;

void dump_rank(int steps, int tecplot, int ascii)
{
    System s1;
    LBM l1(MPI_COMM_WORLD, s1.sx, s1.sy, s1.sz, s1.tau, s1.rho0, s1.u0);
    l1.Initialize();
    for (int it = 1; it <= steps; ++it) {
        l1.Collision();
        l1.Streaming();
        if (it % s1.inter == 0) {
            double mass, px, py, pz, ke;
            l1.Conserved(mass, px, py, pz, ke);
            if (l1.me == 0)
                printf("cons  step %6d | mass %.15e | px %.15e | py %.15e | pz %.15e | ke %.15e\n", it, mass, px, py,
                       pz, ke);
        }
    }
    // this rank's block of the whole lattice
    for (int a = 0; a < 27; ++a)
        for (int i = 0; i < l1.l_l[0]; ++i)
            for (int j = 0; j < l1.l_l[1]; ++j)
                for (int k = 0; k < l1.l_l[2]; ++k)
                    g_field[(((size_t)a * g_gx + l1.x_lo + i) * g_gy + l1.y_lo + j) * g_gz + l1.z_lo + k] =
                        l1.f(a, i + l1.l_s[0], j + l1.l_s[1], k + l1.l_s[2]);
    if (tecplot >= 0 || ascii >= 0) l1.ComputeMacroscopic();
    if (tecplot >= 0) l1.MPIoutput(tecplot);
    if (ascii >= 0) l1.Output(ascii);
    MPI_Barrier(MPI_COMM_WORLD);
}

int usage()
{
    std::fprintf(stderr, "usage: imexref [--ranks N] [--threads T] main\n"
                         "       imexref [--ranks N] [--threads T] dump STEPS FILE [--tecplot K] [--ascii K]\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv)
{
    int ranks = 1, threads = 0, a = 1;
    while (a + 1 < argc && argv[a][0] == '-' && argv[a][1] == '-') {
        if (!std::strcmp(argv[a], "--ranks")) ranks = std::atoi(argv[a + 1]);
        else if (!std::strcmp(argv[a], "--threads")) threads = std::atoi(argv[a + 1]);
        else return usage();
        a += 2;
    }
    if (a >= argc || ranks < 1 || threads < 0) return usage();
    const std::string mode = argv[a];
    imexref_set_world(ranks, threads);
    std::vector<std::thread> pool;
    if (mode == "main") {
        char* args[] = {argv[0], nullptr};
        for (int r = 0; r < ranks; ++r)
            pool.emplace_back([r, &args] {
                imexref_set_rank(r);
                imexref_main(1, args);
            });
        for (auto& t : pool) t.join();
        return 0;
    }
    if (mode != "dump" || a + 2 >= argc) return usage();
    const int steps = std::atoi(argv[a + 1]);
    const char* out = argv[a + 2];
    int tecplot = -1, ascii = -1;
    for (int b = a + 3; b + 1 < argc; b += 2) {
        if (!std::strcmp(argv[b], "--tecplot")) tecplot = std::atoi(argv[b + 1]);
        else if (!std::strcmp(argv[b], "--ascii")) ascii = std::atoi(argv[b + 1]);
        else return usage();
    }
    {
        System deck;  // the whole lattice's size, from ./input.in
        g_gx = deck.sx;
        g_gy = deck.sy;
        g_gz = deck.sz;
    }
    g_field.assign((size_t)27 * g_gx * g_gy * g_gz, 0.0);
    for (int r = 0; r < ranks; ++r)
        pool.emplace_back([r, steps, tecplot, ascii] {
            imexref_set_rank(r);
            dump_rank(steps, tecplot, ascii);
        });
    for (auto& t : pool) t.join();
    FILE* fp = std::fopen(out, "wb");
    if (!fp || std::fwrite(g_field.data(), sizeof(double), g_field.size(), fp) != g_field.size()) {
        std::fprintf(stderr, "imexref: cannot write %s\n", out);
        return 1;
    }
    std::fclose(fp);
    return 0;
}
