/*
 * CPU ORACLE - test infrastructure only, never part of the product path.
 *
 * A plain-C, FP64 restatement of the reference IMEXLBM single-rank time step
 * (Maccchiatooo/IMEXLBM).  Tests, the smoke check and the benchmark's CPU
 * baseline call it as the checker; the CUDA library never links or calls it.
 *
 * What is restated, and from where (paths relative to the reference project):
 *   deck + derived tau        src/System.cpp:22-28   (Re is an int, System.hpp:18)
 *   lattice tables            src/lbm.cpp:3-35       (pi = 3.1415926, not M_PI)
 *   Taylor-Green init + feq   src/lbm.cpp:78-108
 *   fused BGK collision       src/lbm.cpp:131-166
 *   pull streaming            src/lbm.cpp:168-207
 *   conserved diagnostics     src/lbm.cpp:266-306
 * On one rank the reference's ghost-layer halo (src/mpi_view_transfer.cpp:
 * 260-456: faces, then edges, then corners, all self-channels) makes every
 * ghost cell a periodic image of an interior cell, so streaming here reads
 * the periodic image directly.
 *
 * Floating-point expressions keep the reference's evaluation order, and the
 * file is compiled with -ffp-contract=off so x86 and aarch64 hosts give the
 * same bits (the reference's x86 CPU build has no FMA either).
 *
 * Layout: f[q][nx][ny][nz], z fastest, interior cells only (the reference's
 * LayoutRight View with its 3 ghost layers stripped).
 *
 * Parity pin: the reference ships no field dumps; its only known answers are
 * the 32^3 kinetic-energy trajectory 9.852 -> 10.219 -> 9.889 after steps 1-3
 * and the mass / momentum invariants (tests/regression.sh:29,41-42).  The
 * CPU test suite checks this oracle against those values.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Q 27
#define ORACLE_PI 3.1415926 /* src/lbm.cpp:3 */

/* src/lbm.cpp:9-19 */
static const double W[Q] = {
    8.0 / 27.0,
    2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0,
    1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0,
    1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0,
    1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0, 1.0 / 54.0,
    1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0,
    1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0};

/* src/lbm.cpp:20-30, same direction order */
static const int E[Q][3] = {
    {0, 0, 0},
    {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},
    {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
    {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1},
    {1, 1, 1}, {-1, -1, -1}, {1, -1, 1}, {-1, 1, -1},
    {1, 1, -1}, {-1, -1, 1}, {1, -1, -1}, {-1, 1, 1}};

static int g_threads = 1;

void oracle_set_threads(int n) { g_threads = n > 0 ? n : 1; }

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

double oracle_weight(int a) { return (a >= 0 && a < Q) ? W[a] : 0.0; }
int oracle_velocity(int a, int d) { return (a >= 0 && a < Q && d >= 0 && d < 3) ? E[a][d] : 0; }

static inline size_t idx(int a, int i, int j, int k, int nx, int ny, int nz)
{
    return (((size_t)a * nx + i) * ny + j) * nz + k;
}

/* --------------------------------------------------------------------------
 * Deck: nine numbers read the way std::istream >> does in System.cpp:22-24
 * (rho0 R Re / u0 Time inter / sx sy sz, Re/Time/inter/sx/sy/sz are ints).
 * An int field stops at the first non-digit, exactly as operator>>(int&).
 * Returns 0 on success, -1 when a field is missing or malformed.
 * ------------------------------------------------------------------------ */
typedef struct
{
    double rho0, R, u0;
    int Re, Time, inter, sx, sy, sz;
    double cs2, cs, Ma, miu, tau;
} oracle_deck;

static const char *skip_ws(const char *s)
{
    while (*s && isspace((unsigned char)*s)) ++s;
    return s;
}

static int read_int(const char **ps, int *out)
{
    const char *s = skip_ws(*ps);
    const char *b = s;
    if (*s == '+' || *s == '-') ++s;
    if (!isdigit((unsigned char)*s)) return -1;
    while (isdigit((unsigned char)*s)) ++s;
    char buf[64];
    size_t n = (size_t)(s - b);
    if (n >= sizeof buf) return -1;
    memcpy(buf, b, n);
    buf[n] = 0;
    *out = (int)strtol(buf, NULL, 10);
    *ps = s;
    return 0;
}

static int read_double(const char **ps, double *out)
{
    const char *s = skip_ws(*ps);
    const char *b = s;
    int digits = 0;
    if (*s == '+' || *s == '-') ++s;
    while (isdigit((unsigned char)*s)) { ++s; ++digits; }
    if (*s == '.') { ++s; while (isdigit((unsigned char)*s)) { ++s; ++digits; } }
    if (!digits) return -1;
    if (*s == 'e' || *s == 'E')
    {
        const char *t = s + 1;
        if (*t == '+' || *t == '-') ++t;
        if (isdigit((unsigned char)*t)) { while (isdigit((unsigned char)*t)) ++t; s = t; }
    }
    char buf[128];
    size_t n = (size_t)(s - b);
    if (n >= sizeof buf) return -1;
    memcpy(buf, b, n);
    buf[n] = 0;
    *out = strtod(buf, NULL);
    *ps = s;
    return 0;
}

int oracle_deck_parse(const char *text, oracle_deck *d)
{
    const char *s = text;
    memset(d, 0, sizeof *d);
    if (read_double(&s, &d->rho0) || read_double(&s, &d->R) || read_int(&s, &d->Re) ||
        read_double(&s, &d->u0) || read_int(&s, &d->Time) || read_int(&s, &d->inter) ||
        read_int(&s, &d->sx) || read_int(&s, &d->sy) || read_int(&s, &d->sz))
        return -1;
    /* System.cpp:13-14, 26-28, left-to-right as written */
    d->cs2 = 1.0 / 3.0;
    d->cs = sqrt(d->cs2);
    d->Ma = d->u0 / d->cs;
    d->miu = d->rho0 * d->u0 * d->sx / 2.0 / 3.1415926 / d->Re;
    d->tau = d->u0 * d->sx / d->Re / d->cs2 / 2.0 / 3.1415926;
    return 0;
}

/* --------------------------------------------------------------------------
 * Initialisation, src/lbm.cpp:78-108 (node coordinate of interior cell i is
 * (i - ghost + x_lo) = i on one rank).
 * ------------------------------------------------------------------------ */
void oracle_init(int nx, int ny, int nz, double rho0, double u0, double *f)
{
    const double cs2 = 1.0 / 3.0; /* lbm.hpp:182 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
            {
                const double xx = (double)i / (double)nx * 2.0 * ORACLE_PI;
                const double yy = (double)j / (double)ny * 2.0 * ORACLE_PI;
                const double zz = (double)k / (double)nz * 2.0 * ORACLE_PI;
                const double sx = sin(xx), cx = cos(xx);
                const double sy = sin(yy), cy = cos(yy);
                const double cz = cos(zz);
                const double u = u0 * sx * cy * cz;
                const double v = -u0 * cx * sy * cz;
                const double w = 0.0;
                const double p = rho0 * cs2 +
                                 rho0 * u0 * u0 / 16.0 * (cos(2.0 * xx) + cos(2.0 * yy)) *
                                     (cos(2.0 * zz) + 2.0);
                for (int a = 0; a < Q; ++a)
                {
                    const double edu = E[a][0] * u + E[a][1] * v + E[a][2] * w;
                    const double udu = u * u + v * v + w * w;
                    f[idx(a, i, j, k, nx, ny, nz)] =
                        W[a] * (3.0 * p + 3.0 * edu + 4.5 * edu * edu - 1.5 * udu);
                }
            }
}

/* --------------------------------------------------------------------------
 * BGK collision in place, src/lbm.cpp:131-166.
 * ------------------------------------------------------------------------ */
void oracle_collide(int nx, int ny, int nz, double tau0, double *f)
{
    const double inv_tau = 1.0 / (tau0 + 0.5);
    const size_t plane = (size_t)nx * ny * nz;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
            {
                const size_t c = ((size_t)i * ny + j) * nz + k;
                double fl[Q];
                double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
                for (int a = 0; a < Q; ++a)
                {
                    const double fv = f[a * plane + c];
                    fl[a] = fv;
                    pl += fv;
                    ul += fv * E[a][0];
                    vl += fv * E[a][1];
                    wl += fv * E[a][2];
                }
                const double u = ul, v = vl, w = wl;
                const double pp = pl * (1.0 / 3.0);
                const double udu = u * u + v * v + w * w;
                for (int a = 0; a < Q; ++a)
                {
                    const double edu = E[a][0] * u + E[a][1] * v + E[a][2] * w;
                    const double feq = W[a] * (3.0 * pp + 3.0 * edu + 4.5 * edu * edu - 1.5 * udu);
                    f[a * plane + c] = fl[a] - (fl[a] - feq) * inv_tau;
                }
            }
}

/* --------------------------------------------------------------------------
 * Pull streaming, src/lbm.cpp:186-197: ft(a, x) = f(a, x - e_a), with the
 * one-rank halo being the periodic image.  Writes ft; the caller swaps.
 * ------------------------------------------------------------------------ */
void oracle_stream(int nx, int ny, int nz, const double *f, double *ft)
{
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int a = 0; a < Q; ++a)
        for (int i = 0; i < nx; ++i)
        {
            const int si = (i - E[a][0] + nx) % nx;
            for (int j = 0; j < ny; ++j)
            {
                const int sj = (j - E[a][1] + ny) % ny;
                const double *src = f + idx(a, si, sj, 0, nx, ny, nz);
                double *dst = ft + idx(a, i, j, 0, nx, ny, nz);
                for (int k = 0; k < nz; ++k)
                    dst[k] = src[(k - E[a][2] + nz) % nz];
            }
        }
}

/* One reference time step: Collision() then Streaming() (src/main.cpp:43,61),
 * then std::swap(f, ft) (src/lbm.cpp:206): the result lands back in f. */
void oracle_step(int nx, int ny, int nz, double tau0, double *f, double *ft, int nsteps)
{
    const size_t n = (size_t)Q * nx * ny * nz;
    for (int s = 0; s < nsteps; ++s)
    {
        oracle_collide(nx, ny, nz, tau0, f);
        oracle_stream(nx, ny, nz, f, ft);
        memcpy(f, ft, n * sizeof(double));
    }
}

/* Collide + stream without the copy back: result in ft (bench timing). */
void oracle_step_pingpong(int nx, int ny, int nz, double tau0, double *f, double *ft)
{
    oracle_collide(nx, ny, nz, tau0, f);
    oracle_stream(nx, ny, nz, f, ft);
}

/* --------------------------------------------------------------------------
 * Conserved diagnostics, src/lbm.cpp:266-306: mass = sum f, momentum =
 * sum f e, ke = 0.5 sum |u|^2 with u = sum_a f_a e_a per cell.  Cells are
 * summed serially in (i, j, k) order.
 * ------------------------------------------------------------------------ */
void oracle_conserved(int nx, int ny, int nz, const double *f, double out[5])
{
    const size_t plane = (size_t)nx * ny * nz;
    double m = 0.0, mx = 0.0, my = 0.0, mz = 0.0, ek = 0.0;
    for (size_t c = 0; c < plane; ++c)
    {
        double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
        for (int a = 0; a < Q; ++a)
        {
            const double fv = f[a * plane + c];
            pl += fv;
            ul += fv * E[a][0];
            vl += fv * E[a][1];
            wl += fv * E[a][2];
        }
        m += pl;
        mx += ul;
        my += vl;
        mz += wl;
        ek += 0.5 * (ul * ul + vl * vl + wl * wl);
    }
    out[0] = m;
    out[1] = mx;
    out[2] = my;
    out[3] = mz;
    out[4] = ek;
}

/* Per-cell macroscopic fields, src/lbm.cpp:213-240 (p = sum f / 3, u = sum f e). */
void oracle_macroscopic(int nx, int ny, int nz, const double *f,
                        double *p, double *u, double *v, double *w)
{
    const size_t plane = (size_t)nx * ny * nz;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (long long cc = 0; cc < (long long)plane; ++cc)
    {
        const size_t c = (size_t)cc;
        double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
        for (int a = 0; a < Q; ++a)
        {
            const double fv = f[a * plane + c];
            pl += fv;
            ul += fv * E[a][0];
            vl += fv * E[a][1];
            wl += fv * E[a][2];
        }
        p[c] = pl * (1.0 / 3.0);
        u[c] = ul;
        v[c] = vl;
        w[c] = wl;
    }
}
