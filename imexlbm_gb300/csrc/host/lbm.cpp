// C++ facade over the C ABI: class System and struct LBM (see lbm.hpp).
#include "lbm.hpp"

#include <iostream>

namespace {

void throw_on(int rc, const imex_lattice* h)
{
    if (rc != IMEX_OK) throw imex::Error(rc, imex_last_error(h));
}

}  // namespace

System::System() { load("input.in"); }

System::System(const char* path) { load(path); }

void System::load(const char* path)
{
    imex_deck d;
    throw_on(imex_deck_read(path, &d), nullptr);
    rho0 = d.rho0;
    R = d.R;
    Re = d.Re;
    u0 = d.u0;
    Time = d.Time;
    inter = d.inter;
    sx = d.sx;
    sy = d.sy;
    sz = d.sz;
    cs2 = d.cs2;
    cs = d.cs;
    Ma = d.Ma;
    miu = d.miu;
    tau = d.tau;
}

// Same banner as the reference's System::Monitor (src/System.cpp:31-44).
void System::Monitor()
{
    std::cout << "============================" << std::endl
              << "3D Taylor-Green Vortex" << std::endl
              << "Re    = " << Re << std::endl
              << "Ma    = " << Ma << std::endl
              << "rho   = " << rho0 << std::endl
              << "miu   = " << miu << std::endl
              << "tau   = " << tau << std::endl
              << "Time  = " << Time << std::endl
              << "inter = " << inter << std::endl
              << "nx,ny,nz = " << sx << " " << sy << " " << sz << std::endl
              << "============================" << std::endl;
}

LBM::LBM(int sx, int sy, int sz, double& tau, double& rho0_, double& u0_, int precision)
    : glx(sx), gly(sy), glz(sz), rho0(rho0_), cs2(1.0 / 3.0), tau0(tau), u0(u0_)
{
    throw_on(imex_create(sx, sy, sz, tau, rho0_, u0_, precision, &h_), nullptr);
}

LBM::~LBM() { imex_destroy(h_); }

void LBM::check(int rc) const { throw_on(rc, h_); }

void LBM::Initialize() { check(imex_initialize(h_)); }
void LBM::Collision() { check(imex_collision(h_)); }
void LBM::Streaming() { check(imex_streaming(h_)); }
void LBM::Step(int n) { check(imex_step(h_, n)); }
void LBM::fence() { check(imex_synchronize(h_)); }

void LBM::ComputeMacroscopic(double* p, double* u, double* v, double* w) { check(imex_macroscopic(h_, p, u, v, w)); }

void LBM::MPIoutput(int n) { check(imex_write_tecplot(h_, nullptr, n)); }
void LBM::Output(int n) { check(imex_write_output(h_, nullptr, n)); }

void LBM::profile_enable(bool on) { check(imex_profile_enable(h_, on ? 1 : 0)); }

void LBM::profile_read(imex_phase_stats out[IMEX_NPHASE], bool reset) { check(imex_profile_read(h_, out, reset ? 1 : 0)); }

void LBM::Conserved(double& mass, double& mom_x, double& mom_y, double& mom_z, double& ke)
{
    // A diverged run (NaN/Inf) still reports its values, as the reference
    // prints them; every other failure throws.
    double out[5];
    const int rc = imex_conserved(h_, out);
    if (rc != IMEX_ERR_NONFINITE) check(rc);
    mass = out[0];
    mom_x = out[1];
    mom_y = out[2];
    mom_z = out[3];
    ke = out[4];
}
