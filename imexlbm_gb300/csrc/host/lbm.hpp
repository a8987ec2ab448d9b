// C++ facade with the reference's class System / struct LBM call surface
// (src/System.hpp:7-19, src/lbm.hpp:113-211), implemented on the C ABI in
// include/imexlbm.h.  A driver written against the reference's main.cpp
// keeps its shape:
//
//     System s1;                       // reads ./input.in
//     LBM l1(s1.sx, s1.sy, s1.sz, s1.tau, s1.rho0, s1.u0);
//     l1.Initialize();
//     for (...) { l1.Collision(); l1.Streaming(); ... l1.Conserved(m, px, py, pz, ke); }
//
// Differences, all on error paths: the reference aborts on a missing deck
// and relies on MPI/Kokkos fatal errors; here every failure throws
// imex::Error carrying the library's status code and message.  One process
// drives one lattice on one GPU; the MPI communicator argument of the
// reference's constructor is accepted and ignored (rank 0 of 1).
#pragma once

#include <stdexcept>
#include <string>

#include "imexlbm.h"

namespace imex {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

}  // namespace imex

class System {
public:
    System();                         // parse ./input.in (System.cpp:11-29)
    explicit System(const char* path);
    void Monitor();                   // System.cpp:31-44

    int sx, sy, sz;
    int Time, inter;
    double miu, u0, R, rho0, Ma, tau;
    int Re;
    double cs2, cs;

private:
    void load(const char* path);
};

struct LBM {
    int nranks = 1;
    int me = 0;
    int glx, gly, glz;
    double rho0, mu = 0.0, cs2, tau0, u0;

    LBM(int sx, int sy, int sz, double& tau, double& rho0, double& u0, int precision = IMEX_F64);
    // Same argument list as the reference (lbm.hpp:179): the communicator is
    // ignored: one lattice per process, on one GPU.
    template <class Comm>
    LBM(Comm, int sx, int sy, int sz, double& tau, double& rho0, double& u0, int precision = IMEX_F64)
        : LBM(sx, sy, sz, tau, rho0, u0, precision)
    {
    }
    ~LBM();
    LBM(const LBM&) = delete;
    LBM& operator=(const LBM&) = delete;

    void Initialize();
    void Collision();
    void Streaming();
    // n reference steps (Collision then Streaming each) in one call: the same
    // numbers, run as one fixed-point run on the float64 engine (imex_step).
    // Not in the reference's struct.
    void Step(int n);
    void ComputeMacroscopic(double* p, double* u, double* v, double* w);
    void Conserved(double& mass, double& mom_x, double& mom_y, double& mom_z, double& ke);
    void MPIoutput(int n);  // lbm.cpp:307-598: writes output<n>.plt
    void Output(int n);     // lbm.cpp:606-636: writes output<n>0.dat (f(0) as text)
    void fence();
    // per-phase device time of this lattice's kernels (imex_profile_*)
    void profile_enable(bool on);
    void profile_read(imex_phase_stats out[IMEX_NPHASE], bool reset);

    imex_lattice* handle() const { return h_; }

private:
    imex_lattice* h_ = nullptr;
    void check(int rc) const;
};
