// Field output and the min/max report diagnostics:
//   imex_minmax_uvwp      the "minmax_uvwp" reduction of LBM::MPIoutput
//                         (src/lbm.cpp:351-372)
//   imex_write_output     LBM::Output on one rank (src/lbm.cpp:606-636): the
//                         ASCII dump of f(0)
//   imex_write_tecplot    LBM::MPIoutput on one rank (src/lbm.cpp:307-598):
//                         a binary Tecplot file of x, y, z, u, v, w, p
//   imex_checkpoint_save  the handle's raw device state to a file, and
//   imex_checkpoint_load  back (no reference counterpart)
//
// One kernel serves the min/max and the Tecplot file: per cell it forms p = sum f / 3 and
// u = sum f e (the ComputeMacroscopic moments, src/lbm.cpp:218-236, pulled
// through a pending streaming), reduces their minima and maxima, and - for
// the file - writes the four fields transposed to the file's x-fastest
// (Fortran) order through a shared-memory tile, so both the reads along z
// and the writes along x are coalesced.  The file is then streamed to disk
// in chunks through two pinned host buffers, copy of one chunk overlapping
// the write of the other.
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "kernels_common.cuh"
#include "lattice_internal.hpp"
#include "lowp_math.cuh"

namespace imex {
namespace {

constexpr int kTile = 32;         // cells per tile side (x and z)
constexpr int kFieldThreads = 256;  // 8 warps, 4 tile rows each

template <int P>
struct Src {  // float32 / float16-deviation storage
    using T = typename lowp::Storage<P>::T;
    static __device__ __forceinline__ double get(const T* p, int a) { return lowp::Storage<P>::to_f64(*p, a); }
};
template <>
struct Src<IMEX_F64> {
    using T = double;
    static __device__ __forceinline__ double get(const double* p, int) { return __ldg(p); }
};

// Order-preserving map of a non-NaN double to an unsigned key, so that
// atomicMax / atomicMin on keys are max / min on the doubles.
__host__ __device__ inline unsigned long long order_key(double d)
{
#ifdef __CUDA_ARCH__
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
#else
    unsigned long long b;
    std::memcpy(&b, &d, 8);
#endif
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

inline double order_unkey(unsigned long long k)
{
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

// One (32 z) x (32 x) tile of one y row per block.  mm[0..3] = max of u, v,
// w, p and mm[4..7] = their min, as order keys; NaN values are skipped, as
// the reference's `if (u > umx)` comparisons skip them.  out (optional) =
// u, v, w, p blocks of ncells doubles each, index x + nx (y + ny z).
template <int P, bool PULL>
__global__ void __launch_bounds__(kFieldThreads) k_fields(const typename Src<P>::T* __restrict__ src, Geom g,
                                                          double* __restrict__ out, unsigned long long* __restrict__ mm)
{
    __shared__ double tile[4][kTile][kTile + 1];
    const int k0 = blockIdx.x * kTile, i0 = blockIdx.y * kTile, j = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double mx[4] = {-DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX};
    double mn[4] = {DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX};
    for (int r = warp; r < kTile; r += kFieldThreads / 32) {
        const int i = i0 + r, k = k0 + lane;
        if (i >= g.nx || k >= g.nz) continue;
        const PullIndex pi(g, i, j, k, PULL);
        double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
#pragma unroll
        for (int a = 0; a < kQ; ++a) {
            const double fv = Src<P>::get(src + pi.at_dyn(g, a), a);
            pl += fv;
            if (ex(a, 0) == 1) ul += fv;
            if (ex(a, 0) == -1) ul -= fv;
            if (ex(a, 1) == 1) vl += fv;
            if (ex(a, 1) == -1) vl -= fv;
            if (ex(a, 2) == 1) wl += fv;
            if (ex(a, 2) == -1) wl -= fv;
        }
        const double val[4] = {ul, vl, wl, pl * (1.0 / 3.0)};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tile[c][r][lane] = val[c];
            if (val[c] > mx[c]) mx[c] = val[c];
            if (val[c] < mn[c]) mn[c] = val[c];
        }
    }
    if (out) {
        __syncthreads();
        for (int r = warp; r < kTile; r += kFieldThreads / 32) {
            const int k = k0 + r, i = i0 + lane;
            if (k >= g.nz || i >= g.nx) continue;
            const size_t o = ((size_t)k * g.ny + j) * g.nx + i;
#pragma unroll
            for (int c = 0; c < 4; ++c) out[c * g.plane + o] = tile[c][lane][r];
        }
    }
    // warp, then block, then one atomic per value and block
    __shared__ double red[kFieldThreads / 32][8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double a = __shfl_down_sync(0xffffffffu, mx[c], o);
            const double b = __shfl_down_sync(0xffffffffu, mn[c], o);
            if (a > mx[c]) mx[c] = a;
            if (b < mn[c]) mn[c] = b;
        }
        if (lane == 0) {
            red[warp][c] = mx[c];
            red[warp][4 + c] = mn[c];
        }
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        const int c = threadIdx.x;
        double v = red[0][c];
        for (int w = 1; w < kFieldThreads / 32; ++w) {
            const double x = red[w][c];
            if (c < 4 ? x > v : x < v) v = x;
        }
        if (c < 4) atomicMax(mm + c, order_key(v));
        else atomicMin(mm + c, order_key(v));
    }
}

template <int P>
cudaError_t launch_fields_p(bool pull, const void* src, const Geom& g, double* out, unsigned long long* mm, cudaStream_t s)
{
    const dim3 grid((g.nz + kTile - 1) / kTile, (g.nx + kTile - 1) / kTile, g.ny);
    using T = typename Src<P>::T;
    if (pull)
        k_fields<P, true><<<grid, kFieldThreads, 0, s>>>(static_cast<const T*>(src), g, out, mm);
    else
        k_fields<P, false><<<grid, kFieldThreads, 0, s>>>(static_cast<const T*>(src), g, out, mm);
    return cudaGetLastError();
}

cudaError_t launch_fields(int prec, bool pull, const void* src, const Geom& g, double* out, unsigned long long* mm,
                          cudaStream_t s)
{
    switch (prec) {
    case IMEX_F64: return launch_fields_p<IMEX_F64>(pull, src, g, out, mm, s);
    case IMEX_F32: return launch_fields_p<IMEX_F32>(pull, src, g, out, mm, s);
    case IMEX_F16DEV: return launch_fields_p<IMEX_F16DEV>(pull, src, g, out, mm, s);
    default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------- host side --
int fail(imex_lattice* h, int code, const std::string& msg) { return lattice_fail(h, code, msg); }

int cuda_fail(imex_lattice* h, cudaError_t e, const std::string& what)
{
    cudaGetLastError();
    return fail(h, IMEX_ERR_CUDA, what + ": " + cudaGetErrorString(e));
}

int ready(imex_lattice* h, const char* what)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": null handle");
    if (h->tag == kUninit) return fail(h, IMEX_ERR_STATE, std::string(what) + ": lattice not initialised");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, what);
    return IMEX_OK;
}

// Run the field kernel; minmax[8] on return, the fields (if out) queued.
int run_fields(imex_lattice* h, double* out, unsigned long long* d_mm, double minmax[8], const char* what)
{
    unsigned long long keys[8];
    for (int c = 0; c < 4; ++c) {
        keys[c] = order_key(-DBL_MAX);
        keys[4 + c] = order_key(DBL_MAX);
    }
    cudaError_t e = cudaMemcpyAsync(d_mm, keys, sizeof keys, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        PhaseScope timed(h->prof, IMEX_PHASE_MACRO, h->stream);
        e = launch_fields(h->precision, h->tag == kPendingStream, h->buf[h->cur], h->g, out, d_mm, h->stream);
    }
    if (e == cudaSuccess) ++h->launches;
    if (e == cudaSuccess) e = cudaMemcpyAsync(keys, d_mm, sizeof keys, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, what);
    for (int c = 0; c < 8; ++c) minmax[c] = order_unkey(keys[c]);
    return IMEX_OK;
}

// Host <-> device streaming of large blocks through two pinned buffers.
struct Pinned {
    void* p[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    size_t cap = 0;
    cudaError_t init(size_t bytes)
    {
        cap = bytes;
        cudaError_t e = cudaSuccess;
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            e = cudaMallocHost(&p[b], cap);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
        }
        return e;
    }
    ~Pinned()
    {
        for (int b = 0; b < 2; ++b) {
            if (p[b]) cudaFreeHost(p[b]);
            if (ev[b]) cudaEventDestroy(ev[b]);
        }
    }
};

constexpr size_t kChunk = 32u << 20;

// Write n bytes of device memory to fp.  Returns 0, or -1 for a file error
// (a CUDA error is returned in *ce).
int device_to_file(const unsigned char* dev, size_t n, FILE* fp, Pinned& pb, cudaStream_t s, cudaError_t* ce)
{
    *ce = cudaSuccess;
    const size_t nchunks = (n + pb.cap - 1) / pb.cap;
    auto issue = [&](size_t c) {
        const size_t off = c * pb.cap, len = std::min(pb.cap, n - off);
        cudaError_t e = cudaMemcpyAsync(pb.p[c & 1], dev + off, len, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaEventRecord(pb.ev[c & 1], s);
        return e;
    };
    if (nchunks && (*ce = issue(0)) != cudaSuccess) return 0;
    for (size_t c = 0; c < nchunks; ++c) {
        if ((*ce = cudaEventSynchronize(pb.ev[c & 1])) != cudaSuccess) return 0;
        if (c + 1 < nchunks && (*ce = issue(c + 1)) != cudaSuccess) return 0;
        const size_t off = c * pb.cap, len = std::min(pb.cap, n - off);
        if (std::fwrite(pb.p[c & 1], 1, len, fp) != len) {
            cudaStreamSynchronize(s);
            return -1;
        }
    }
    return 0;
}

// Read n bytes from fp into device memory; same conventions.
int file_to_device(unsigned char* dev, size_t n, FILE* fp, Pinned& pb, cudaStream_t s, cudaError_t* ce)
{
    *ce = cudaSuccess;
    const size_t nchunks = (n + pb.cap - 1) / pb.cap;
    for (size_t c = 0; c < nchunks; ++c) {
        const size_t off = c * pb.cap, len = std::min(pb.cap, n - off);
        if (c >= 2 && (*ce = cudaEventSynchronize(pb.ev[c & 1])) != cudaSuccess) return 0;  // buffer free again
        if (std::fread(pb.p[c & 1], 1, len, fp) != len) {
            cudaStreamSynchronize(s);
            return -1;
        }
        if ((*ce = cudaMemcpyAsync(dev + off, pb.p[c & 1], len, cudaMemcpyHostToDevice, s)) != cudaSuccess) return 0;
        if ((*ce = cudaEventRecord(pb.ev[c & 1], s)) != cudaSuccess) return 0;
    }
    *ce = cudaStreamSynchronize(s);
    return 0;
}

// Little builder of the binary header.
struct Bytes {
    std::vector<unsigned char> b;
    template <typename T>
    void put(T v)
    {
        const size_t o = b.size();
        b.resize(o + sizeof v);
        std::memcpy(b.data() + o, &v, sizeof v);
    }
    void i32(int v) { put<int32_t>(v); }
    void f32(float v) { put<float>(v); }
    void f64(double v) { put<double>(v); }
};

// The 332-byte header of LBM::MPIoutput (src/lbm.cpp:397-562): Tecplot
// binary version 112, one ordered zone "ZONE 001" of nx*ny*nz nodes, seven
// float64 variables x, y, z, u, v, w, p, solution time n, and the variable
// ranges (x, y, z written as [0, 1]; u, v, w, p from `mm`, min then max).
std::vector<unsigned char> tecplot_header(const Geom& g, int n, const double mm[8])
{
    Bytes h;
    const char magic[8] = {'#', '!', 'T', 'D', 'V', '1', '1', '2'};
    for (char c : magic) h.put<char>(c);
    h.i32(1);  // byte-order integer
    h.i32(0);  // file type: full
    h.i32(0);  // title: empty string
    h.i32(7);  // number of variables
    for (int c : {'x', 'y', 'z', 'u', 'v', 'w', 'p'}) {
        h.i32(c);
        h.i32(0);
    }
    h.f32(299.0f);  // zone marker
    for (int c : {'Z', 'O', 'N', 'E', ' ', '0', '0', '1'}) h.i32(c);
    h.i32(0);
    h.i32(-1);        // parent zone
    h.f64((double)n);  // solution time
    h.i32(0);         // strand (not used)
    h.i32(-1);        // zone colour
    h.i32(0);         // zone type: ordered
    h.i32(0);         // variable location not specified
    h.i32(0);         // no raw face neighbours
    h.i32(0);         // no miscellaneous face connections
    h.i32(g.nx);
    h.i32(g.ny);
    h.i32(g.nz);
    h.i32(0);         // no auxiliary data
    h.f32(357.0f);    // end of header
    h.f32(299.0f);    // data section
    for (int v = 0; v < 7; ++v) h.i32(2);  // float64
    h.i32(0);         // no passive variables
    h.i32(0);         // no shared variables
    h.i32(-1);        // no shared connectivity
    for (int d = 0; d < 3; ++d) {
        h.f64(0.0);
        h.f64(1.0);
    }
    for (int c = 0; c < 4; ++c) {  // mm: max u v w p, then min u v w p
        h.f64(mm[4 + c]);
        h.f64(mm[c]);
    }
    return h.b;
}

// Checkpoint file: this header, then the stored array of the current
// buffer (27 * cells values in the handle's storage type and layout).
struct CkptHeader {
    char magic[8];
    int32_t version, precision, nx, ny, nz, rounding, pending;
    int64_t steps;
    double tau0, rho0, u0;
    uint64_t payload;
};
constexpr char kCkptMagic[8] = {'I', 'M', 'E', 'X', 'C', 'K', 'P', 'T'};

}  // namespace
}  // namespace imex

using namespace imex;

extern "C" {

int imex_minmax_uvwp(imex_lattice* h, double out[8])
{
    int rc = ready(h, "imex_minmax_uvwp");
    if (rc) return rc;
    if (!out) return fail(h, IMEX_ERR_ARG, "imex_minmax_uvwp: null output");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, 8 * sizeof(unsigned long long), h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_minmax_uvwp");
    rc = run_fields(h, nullptr, d, out, "imex_minmax_uvwp");
    cudaFreeAsync(d, h->stream);
    return rc;
}

int imex_write_tecplot(imex_lattice* h, const char* path, int n)
{
    int rc = ready(h, "imex_write_tecplot");
    if (rc) return rc;
    const std::string name = path ? std::string(path) : "output" + std::to_string(n) + ".plt";
    const Geom& g = h->g;
    const size_t nb = h->ncells * sizeof(double);
    double* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, 4 * nb + 8 * sizeof(unsigned long long), h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_write_tecplot: device staging");
    unsigned long long* d_mm = reinterpret_cast<unsigned long long*>(d + 4 * h->ncells);
    double mm[8];
    rc = run_fields(h, d, d_mm, mm, "imex_write_tecplot");
    FILE* fp = rc ? nullptr : std::fopen(name.c_str(), "wb");
    if (!rc && !fp) rc = fail(h, IMEX_ERR_IO, "imex_write_tecplot: cannot open " + name);
    Pinned pb;
    if (!rc && (e = pb.init(std::min(kChunk, std::max<size_t>(nb, 8)))) != cudaSuccess)
        rc = cuda_fail(h, e, "imex_write_tecplot: pinned buffers");
    if (!rc) {
        const std::vector<unsigned char> hdr = tecplot_header(g, n, mm);
        bool ok = std::fwrite(hdr.data(), 1, hdr.size(), fp) == hdr.size();
        // node coordinates (src/lbm.cpp:341-343): index / (extent - 1)
        std::vector<double> line;
        for (int dim = 0; dim < 3 && ok; ++dim) {
            const int ext = dim == 0 ? g.nx : dim == 1 ? g.ny : g.nz;
            const double den = (double)(ext - 1);
            line.resize(g.nx);
            for (int k = 0; k < g.nz && ok; ++k)
                for (int j = 0; j < g.ny && ok; ++j) {
                    for (int i = 0; i < g.nx; ++i) line[i] = (double)(dim == 0 ? i : dim == 1 ? j : k) / den;
                    ok = std::fwrite(line.data(), sizeof(double), g.nx, fp) == (size_t)g.nx;
                }
        }
        if (ok) {
            int io = device_to_file(reinterpret_cast<const unsigned char*>(d), 4 * nb, fp, pb, h->stream, &e);
            if (e != cudaSuccess) rc = cuda_fail(h, e, "imex_write_tecplot: copy");
            ok = io == 0;
        }
        if (std::fclose(fp) != 0) ok = false;
        fp = nullptr;
        if (!rc && !ok) rc = fail(h, IMEX_ERR_IO, "imex_write_tecplot: write to " + name + " failed");
    }
    if (fp) std::fclose(fp);
    cudaFreeAsync(d, h->stream);
    cudaStreamSynchronize(h->stream);
    return rc;
}

int imex_write_output(imex_lattice* h, const char* path, int n)
{
    int rc = ready(h, "imex_write_output");
    if (rc) return rc;
    const std::string name = path ? std::string(path) : "output" + std::to_string(n) + "0.dat";
    const Geom& g = h->g;
    // f(0), the rest population: streaming does not move it, so a pending
    // streaming changes nothing here
    std::vector<double> f0(h->ncells);
    cudaError_t e = cudaSuccess;
    if (h->precision == IMEX_F64) {
        e = cudaMemcpyAsync(f0.data(), h->buf[h->cur], h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    } else {
        double* d = nullptr;
        e = cudaMallocAsync(&d, (size_t)kQ * h->ncells * sizeof(double), h->stream);
        if (e == cudaSuccess) e = launch_to_f64(h->precision, false, h->buf[h->cur], g, d, h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(f0.data(), d, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (d) cudaFreeAsync(d, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_write_output: copy");
    FILE* fp = std::fopen(name.c_str(), "wb");
    if (!fp) return fail(h, IMEX_ERR_IO, "imex_write_output: cannot open " + name);
    // src/lbm.cpp:606-627: a header, then one line "x y z f" per cell with x
    // fastest, f fixed with 8 decimals (std::fixed, setprecision(8))
    std::string out = "variables=x,y,z,f\n";
    out += "zone I=" + std::to_string(g.nx) + ",J=" + std::to_string(g.ny) + ",K=" + std::to_string(g.nz) + "\n";
    bool ok = true;
    char line[96];
    for (int k = 0; k < g.nz && ok; ++k)
        for (int j = 0; j < g.ny && ok; ++j) {
            for (int i = 0; i < g.nx; ++i) {
                const int len = std::snprintf(line, sizeof line, "%d %d %d %.8f\n", i, j, k,
                                              f0[((size_t)i * g.ny + j) * g.nz + k]);
                out.append(line, (size_t)len);
            }
            if (out.size() > (1u << 22)) {
                ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
                out.clear();
            }
        }
    if (ok && !out.empty()) ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
    if (std::fclose(fp) != 0) ok = false;
    return ok ? IMEX_OK : fail(h, IMEX_ERR_IO, "imex_write_output: write to " + name + " failed");
}

int imex_checkpoint_save(imex_lattice* h, const char* path)
{
    int rc = ready(h, "imex_checkpoint_save");
    if (rc) return rc;
    if (!path) return fail(h, IMEX_ERR_ARG, "imex_checkpoint_save: null path");
    CkptHeader c{};
    std::memcpy(c.magic, kCkptMagic, 8);
    c.version = 1;
    c.precision = h->precision;
    c.nx = h->g.nx;
    c.ny = h->g.ny;
    c.nz = h->g.nz;
    c.rounding = h->cf32.sr ? IMEX_ROUND_STOCHASTIC : IMEX_ROUND_NEAREST;
    c.pending = h->tag == kPendingStream;
    c.steps = h->steps;
    c.tau0 = h->tau0;
    c.rho0 = h->rho0;
    c.u0 = h->u0;
    c.payload = (uint64_t)kQ * h->ncells * lattice_elem_size(h->precision);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(h, IMEX_ERR_IO, std::string("imex_checkpoint_save: cannot open ") + path);
    Pinned pb;
    cudaError_t e = pb.init(std::min<size_t>(kChunk, c.payload));
    bool ok = std::fwrite(&c, sizeof c, 1, fp) == 1;
    int io = 0;
    if (e == cudaSuccess && ok)
        io = device_to_file(static_cast<const unsigned char*>(h->buf[h->cur]), c.payload, fp, pb, h->stream, &e);
    ok = ok && io == 0;
    if (std::fclose(fp) != 0) ok = false;
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_checkpoint_save");
    if (!ok) return fail(h, IMEX_ERR_IO, std::string("imex_checkpoint_save: write to ") + path + " failed");
    return IMEX_OK;
}

int imex_checkpoint_load(imex_lattice* h, const char* path)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_checkpoint_load: null handle");
    if (!path) return fail(h, IMEX_ERR_ARG, "imex_checkpoint_load: null path");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_checkpoint_load");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(h, IMEX_ERR_IO, std::string("imex_checkpoint_load: cannot open ") + path);
    CkptHeader c{};
    const uint64_t payload = (uint64_t)kQ * h->ncells * lattice_elem_size(h->precision);
    if (std::fread(&c, sizeof c, 1, fp) != 1 || std::memcmp(c.magic, kCkptMagic, 8) != 0 || c.version != 1) {
        std::fclose(fp);
        return fail(h, IMEX_ERR_IO, std::string("imex_checkpoint_load: ") + path + " is not a checkpoint");
    }
    if (c.nx != h->g.nx || c.ny != h->g.ny || c.nz != h->g.nz || c.precision != h->precision || c.payload != payload ||
        c.steps < 0 || (c.rounding != IMEX_ROUND_NEAREST && c.rounding != IMEX_ROUND_STOCHASTIC)) {
        std::fclose(fp);
        return fail(h, IMEX_ERR_ARG, "imex_checkpoint_load: the checkpoint's lattice size or precision differs");
    }
    Pinned pb;
    e = pb.init(std::min<size_t>(kChunk, payload));
    int io = 0;
    if (e == cudaSuccess) io = file_to_device(static_cast<unsigned char*>(h->buf[h->cur]), payload, fp, pb, h->stream, &e);
    std::fclose(fp);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_checkpoint_load");
    if (io) {
        h->tag = kUninit;  // the buffer holds part of the file
        return fail(h, IMEX_ERR_IO, std::string("imex_checkpoint_load: ") + path + " is truncated");
    }
    h->tag = c.pending ? kPendingStream : kExact;
    h->steps = c.steps;
    const int sr = h->precision == IMEX_F16DEV && c.rounding == IMEX_ROUND_STOCHASTIC;
    if (sr != h->cf32.sr && !h->shape_pinned) h->shape_mode = -1;  // shape re-chosen for the rounding mode
    h->cf32.sr = sr;
    return IMEX_OK;
}

}  // extern "C"
