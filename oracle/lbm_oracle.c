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
 *   min/max of u, v, w, p     src/lbm.cpp:351-372
 *   Tecplot output (1 rank)   src/lbm.cpp:307-598
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
 * Parity pin: bit for bit against the reference's own code.  The
 * reference's unmodified src/ C++ files, built against the single-process
 * Kokkos / MPI stand-ins of oracle/refshim and run on 1 to 8 ranks,
 * produce fields whose SHA-256 this oracle reproduces exactly (32^3 and
 * 18x20x22 decks, 20-100 steps), `cons` lines it matches to the rounding of
 * the summation order, and a Tecplot file this writer reproduces byte for
 * byte (tests/golden/reference_runs.json, tests/test_reference_pin.py).
 * It also meets the reference's published known answers: the 32^3
 * kinetic-energy trajectory 9.852 -> 10.219 -> 9.889 after steps 1-3 and
 * the mass / momentum invariants (tests/regression.sh:29,41-42).
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

/* Extremes of u, v, w, p, the "minmax_uvwp" reduction of src/lbm.cpp:351-372:
 * out = {umax, vmax, wmax, pmax, umin, vmin, wmin, pmin}, each reducer
 * starting from Kokkos's Max / Min identity (-DBL_MAX / DBL_MAX) and updated
 * by a strict comparison, so NaN values are never taken. */
void oracle_minmax_uvwp(int nx, int ny, int nz, const double *f, double out[8])
{
    const size_t n = (size_t)nx * ny * nz;
    double *m = (double *)malloc(4 * n * sizeof(double));
    oracle_macroscopic(nx, ny, nz, f, m + 3 * n, m, m + n, m + 2 * n); /* u v w p */
    for (int c = 0; c < 4; ++c)
    {
        double mx = -1.7976931348623157e308, mn = 1.7976931348623157e308;
        for (size_t q = 0; q < n; ++q)
        {
            const double x = m[c * n + q];
            if (x > mx) mx = x;
            if (x < mn) mn = x;
        }
        out[c] = mx;
        out[4 + c] = mn;
    }
    free(m);
}

static void put_i32(FILE *fp, int v) { int32_t x = v; fwrite(&x, 4, 1, fp); }
static void put_f32(FILE *fp, float v) { fwrite(&v, 4, 1, fp); }
static void put_f64(FILE *fp, double v) { fwrite(&v, 8, 1, fp); }

/* LBM::MPIoutput(n) on one rank (src/lbm.cpp:307-598): the header fields in
 * the order the reference writes them (:397-562, 332 bytes), then the
 * blocks x, y, z, u, v, w, p as the one-rank file view lays them out
 * (:564-591: each block the whole lattice in Fortran order, x fastest).
 * Coordinates are (double)i / (nx - 1) (:341-343).  Returns 0, or -1 if the
 * file cannot be written. */
int oracle_write_tecplot(int nx, int ny, int nz, const double *f, int n, const char *path)
{
    const size_t cells = (size_t)nx * ny * nz;
    double mm[8];
    oracle_minmax_uvwp(nx, ny, nz, f, mm);
    double *m = (double *)malloc(4 * cells * sizeof(double));
    oracle_macroscopic(nx, ny, nz, f, m + 3 * cells, m, m + cells, m + 2 * cells);
    FILE *fp = fopen(path, "wb");
    if (!fp)
    {
        free(m);
        return -1;
    }
    fwrite("#!TDV112", 1, 8, fp);
    put_i32(fp, 1);
    put_i32(fp, 0);
    put_i32(fp, 0);
    put_i32(fp, 7);
    const char *names = "xyzuvwp";
    for (int c = 0; c < 7; ++c)
    {
        put_i32(fp, names[c]);
        put_i32(fp, 0);
    }
    put_f32(fp, 299.0f);
    const char *zone = "ZONE 001";
    for (int c = 0; c < 8; ++c)
        put_i32(fp, zone[c]);
    put_i32(fp, 0);
    put_i32(fp, -1);
    put_f64(fp, (double)n);
    put_i32(fp, 0);
    put_i32(fp, -1);
    for (int c = 0; c < 4; ++c)
        put_i32(fp, 0);
    put_i32(fp, nx);
    put_i32(fp, ny);
    put_i32(fp, nz);
    put_i32(fp, 0);
    put_f32(fp, 357.0f);
    put_f32(fp, 299.0f);
    for (int c = 0; c < 7; ++c)
        put_i32(fp, 2);
    put_i32(fp, 0);
    put_i32(fp, 0);
    put_i32(fp, -1);
    for (int c = 0; c < 3; ++c)
    {
        put_f64(fp, 0.0);
        put_f64(fp, 1.0);
    }
    for (int c = 0; c < 4; ++c)
    {
        put_f64(fp, mm[4 + c]);
        put_f64(fp, mm[c]);
    }
    for (int b = 0; b < 7; ++b)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                {
                    double x;
                    if (b == 0) x = (double)i / (nx - 1);
                    else if (b == 1) x = (double)j / (ny - 1);
                    else if (b == 2) x = (double)k / (nz - 1);
                    else x = m[(size_t)(b - 3) * cells + ((size_t)i * ny + j) * nz + k];
                    put_f64(fp, x);
                }
    const int bad = ferror(fp);
    fclose(fp);
    free(m);
    return bad ? -1 : 0;
}
