// C ABI of one resident lattice (include/imexlbm.h).
//
// State machine.  The reference's step is Collision() then Streaming()
// (src/main.cpp:43,61).  The fast kernel here is the fused "pull, then
// collide" K = C(S(.)), so the handle keeps its distributions in one of two
// states:
//   kExact          the device buffer IS the reference's f;
//   kPendingStream  the reference's f is S(buffer): the streaming of the last
//                   step has not been applied yet.
// Transitions (each keeps the reference's meaning for any call sequence):
//   Collision  kExact -> collide in place            -> kExact
//              kPending -> fused K into the other buffer -> kExact
//   Streaming  kExact -> nothing (mark)               -> kPending
//              kPending -> stream into the other buffer -> kPending
// In the steady state Collision launches one fused kernel and Streaming
// launches none.  Readers (Conserved, macroscopic, get_f) pull through S
// when the state is kPending.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "kernels_f64.cuh"
#include "kernels_fx.cuh"
#include "kernels_lowp.cuh"
#include "rows.cuh"
#include "lattice_internal.hpp"
#include "rows_lowp.cuh"

namespace imex {

static thread_local std::string g_thread_err;

int set_thread_error(int code, const std::string& msg)
{
    g_thread_err = msg;
    return code;
}

const char* thread_error() { return g_thread_err.c_str(); }

// Test faults (imex_test_set_fault): read at every launch of a kernel with
// bounded waits; IMEX_TEST_FAULT_NONE in production.
static std::atomic<int> g_fault_kind{IMEX_TEST_FAULT_NONE};
static std::atomic<long long> g_fault_value{0};

int test_fault_kind() { return g_fault_kind.load(std::memory_order_relaxed); }
long long test_fault_value() { return g_fault_value.load(std::memory_order_relaxed); }

WaitCtl make_wait_ctl(unsigned* err)
{
    WaitCtl wc;
    wc.err = err;
    wc.cycles = bulk::kWaitCycles;
    wc.starve_cta = -1;
    if (test_fault_kind() == IMEX_TEST_FAULT_STARVE_STAGE) {
        wc.cycles = test_fault_value();
        wc.starve_cta = 0;
    }
    return wc;
}

int lattice_fail(imex_lattice* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    set_thread_error(code, msg);
    return code;
}

size_t lattice_elem_size(int precision) { return precision == IMEX_F64 ? 8 : precision == IMEX_F32 ? 4 : 2; }

}  // namespace imex

using namespace imex;

namespace {

int fail(imex_lattice* h, int code, const std::string& msg) { return lattice_fail(h, code, msg); }

int cuda_fail(imex_lattice* h, cudaError_t e, const char* what)
{
    cudaGetLastError();  // clear a non-sticky error
    return fail(h, IMEX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define IMEX_CUDA(h, call, what)                           \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
    } while (0)

size_t elem_size(int precision) { return lattice_elem_size(precision); }

bool use_fixed(const imex_lattice* h)
{
    return h->precision == IMEX_F64 && h->fx_ok &&
           (h->engine == IMEX_ENGINE_FIXED || h->engine == IMEX_ENGINE_AUTO);
}

double* dbuf(imex_lattice* h, int which) { return static_cast<double*>(h->buf[which]); }

bool is_lowp(const imex_lattice* h) { return h->precision != IMEX_F64; }

// ------------------------------------------------------------ launch shapes --
// The fused step has two kernels: one thread per cell with direct pulls
// from global memory, and the row-staged kernel (rows.cuh) whose shape is a
// ring depth and a number of resident CTAs per SM.  The autotuner times each
// candidate shape on the handle's own lattice - the fused kernel reads one
// buffer and writes the other, so repeating it changes nothing - and keeps
// the fastest.  Results are cached per (precision, engine, nx, ny, nz).

bool rows_eligible_for(const imex_lattice* h)
{
    if (is_lowp(h)) return rows_lowp_eligible(h->precision, h->g);
    return use_fixed(h) && rows_fx_eligible(h->g);
}

size_t stage_bytes(const imex_lattice* h) { return (size_t)kQ * h->g.nz * elem_size(h->precision); }

// Reduced precision: the smallest direction block (1, 2 or 4 KB) of a stage
// that holds B rows; 0 if none does.
int lowp_dir_bytes(const imex_lattice* h, int B)
{
    const size_t need = (size_t)B * h->g.nz * elem_size(h->precision);
    return need <= 1024 ? 1024 : need <= 2048 ? 2048 : need <= 4096 ? 4096 : 0;
}

std::vector<RowConfig> row_candidates(const imex_lattice* h)
{
    std::vector<RowConfig> out;
    if (!rows_eligible_for(h)) return out;
    if (is_lowp(h)) {
        // (stages, CTAs per SM) per direction block; B from rowslp::item_rows
        const int shapes[][2] = {{2, 2}, {3, 2}, {2, 1}, {3, 1}, {4, 1}};
        const size_t row = (size_t)h->g.nz * elem_size(h->precision);
        for (int dir : {1024, 2048, 4096}) {
            if (row > (size_t)dir) continue;
            const int B = rowslp::item_rows(h->g.ny, h->g.nz, (int)elem_size(h->precision), dir);
            if (lowp_dir_bytes(h, B) != dir) continue;  // same items as a smaller block
            for (const auto& sh : shapes) {
                const size_t smem = rowslp::smem_bytes(dir, sh[0]);
                if (smem > 227 * 1024 || (size_t)sh[1] * (smem + 1024) > 228 * 1024) continue;
                RowConfig rc;
                rc.stages = sh[0];
                rc.ctas_per_sm = sh[1];
                rc.rows = B;
                rc.dir_bytes = dir;
                rc.threads = rowslp::kThreads;
                out.push_back(rc);
            }
        }
        return out;
    }
    const size_t sb = stage_bytes(h);  // one row of all 27 directions
    const size_t per_sm = 227 * 1024;
    const int threads = h->g.nz >= 256 ? 256 : ((h->g.nz + 31) / 32) * 32;
    const int ctas_opts[3] = {1, 2, 4};
    const int stage_opts[3] = {2, 3, 4};
    const int rows_opts[4] = {1, 2, 4, 8};
    for (int c : ctas_opts) {
        if (!is_lowp(h) && c > 2) continue;  // fixed-point engine: 128+ registers per thread
        for (int B : rows_opts) {
            if (h->g.ny % B) continue;
            for (int s : stage_opts) {
                const size_t smem = kRowBarrierBytes + (size_t)s * B * sb;
                if (smem > per_sm / c) continue;
                if ((size_t)s * B * sb < 24 * 1024) continue;  // too little in flight to matter
                RowConfig rc;
                rc.stages = s;
                rc.rows = B;
                rc.ctas_per_sm = c;
                rc.threads = threads;
                out.push_back(rc);
            }
        }
    }
    return out;
}

std::mutex g_tune_lock;
std::map<std::tuple<int, int, int, int, int>, RowConfig> g_tune_cache;

// (precision, engine or rounding mode, nx, ny, nz)
std::tuple<int, int, int, int, int> tune_key(const imex_lattice* h)
{
    return std::make_tuple(h->precision, (use_fixed(h) ? 1 : 0) + 2 * h->cf32.sr, h->g.nx, h->g.ny, h->g.nz);
}

cudaError_t launch_fused_rows(imex_lattice* h, const void* src, void* dst, const RowConfig& rc)
{
    if (is_lowp(h)) return launch_rows_lowp(h->precision, src, dst, h->g, h->cf32, rc, h->d_err, h->stream);
    return launch_rows_fx(static_cast<const double*>(src), static_cast<double*>(dst), h->g, h->fx, h->cf64,
                          h->d_fallback, rc, h->d_err, h->stream);
}

cudaError_t launch_fused_classic(imex_lattice* h, const void* src, void* dst)
{
    if (is_lowp(h)) return launch_step_lowp(h->precision, kModeFused, src, dst, h->g, h->cf32, h->stream);
    if (use_fixed(h))
        return launch_step_fx(kModeFused, static_cast<const double*>(src), static_cast<double*>(dst), h->g, h->fx,
                              h->cf64, h->d_fallback, h->stream);
    return launch_step_f64(kModeFused, static_cast<const double*>(src), static_cast<double*>(dst), h->g, h->cf64,
                           h->stream);
}

// Time the fused step in shape rc (stages 0: classic); milliseconds per launch.
// Milliseconds per launch of `reps` back-to-back fused steps in shape rc
// (stages 0: classic).
int time_shape(imex_lattice* h, const RowConfig& rc, int reps, float* ms)
{
    const void* src = h->buf[h->cur];
    void* dst = h->buf[1 - h->cur];
    cudaEvent_t e0, e1;
    IMEX_CUDA(h, cudaEventCreate(&e0), "cudaEventCreate");
    IMEX_CUDA(h, cudaEventCreate(&e1), "cudaEventCreate");
    cudaError_t e = cudaEventRecord(e0, h->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        e = rc.stages > 0 ? launch_fused_rows(h, src, dst, rc) : launch_fused_classic(h, src, dst);
        if (e == cudaSuccess) h->launches++;
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(h, e, "autotune");
    *ms = t / reps;
    return IMEX_OK;
}

// The one-thread-per-cell shape of the float64 fixed-point engine runs, in
// imex_step's steady state, as k_step_fxs reading and writing X between
// launches (step_fixed_run), not as k_step_fx: time that form, so that the
// row shapes are compared with the kernel that would actually run.  One
// step from the state into the spare buffer gives X on the float64 grid;
// the timed launches read it and write a temporary third buffer, so the
// state is untouched.  Without room for the third buffer it times
// k_step_fx instead.
int time_fixed_run(imex_lattice* h, int reps, float* ms)
{
    const size_t bytes = (size_t)kQ * h->ncells * sizeof(double);
    double* tmp = nullptr;
    if (cudaMallocAsync(&tmp, bytes, h->stream) != cudaSuccess) {
        cudaGetLastError();
        return time_shape(h, RowConfig{}, reps, ms);
    }
    const int n = reps + 2;  // launches 2 .. n-1 read and write X
    double* x = dbuf(h, 1 - h->cur);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMemsetAsync(h->d_fail, 0x7f, sizeof(int), h->stream);
    if (e == cudaSuccess) e = launch_step_fx_run(dbuf(h, h->cur), x, h->g, h->fx, 1, n, h->d_fail, h->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, h->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
        e = launch_step_fx_run(x, tmp, h->g, h->fx, 2 + r, n, h->d_fail, h->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaError_t e2 = cudaFreeAsync(tmp, h->stream);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(h, e, "autotune");
    h->launches += reps + 1;
    *ms = t / reps;
    return IMEX_OK;
}

int check_kernel_error(imex_lattice* h);

// Resources of the two-steps-per-launch kernel (per handle, grown to the
// deepest ring a launch shape asks for): the ticket counter, 2 nx ny row
// flags (zero: no epoch yet) and the ring of `ring` + 2 x-planes.
int ensure_two_step(imex_lattice* h, int ring)
{
    if (h->two_mem && h->two_ring >= ring) return IMEX_OK;
    const size_t rows = (size_t)h->g.nx * h->g.ny;
    const size_t bytes = two_step_ring_values(h->g, ring) * sizeof(unsigned long long);
    const size_t head = (16 + 2 * rows * sizeof(int) + 255) & ~(size_t)255;
    if (h->two_mem) {  // a shallower ring: its flags' epochs are kept by the new one's zeros
        IMEX_CUDA(h, cudaFreeAsync(h->two_mem, h->stream), "cudaFreeAsync");
        h->bytes -= h->two_bytes;
        h->two_mem = nullptr;
    }
    unsigned char* m = nullptr;
    IMEX_CUDA(h, cudaMallocAsync((void**)&m, head + bytes, h->stream), "cudaMallocAsync");
    IMEX_CUDA(h, cudaMemsetAsync(m, 0, head, h->stream), "cudaMemset");
    h->two_mem = m;
    h->two_ring = ring;
    h->two_bytes = head + bytes;
    h->two.counter = reinterpret_cast<unsigned*>(m);
    h->two.flag_a = reinterpret_cast<int*>(m + 16);
    h->two.flag_b = h->two.flag_a + rows;
    h->two.mid = reinterpret_cast<unsigned long long*>(m + head);
    h->two.err = h->d_err;
    h->bytes += h->two_bytes;
    return IMEX_OK;
}

// Steps j, j + 1 of a run in one launch of the two-step kernel, launch
// shape rc (rows: ring depth, ctas_per_sm: resident CTAs).
cudaError_t launch_two(imex_lattice* h, const RowConfig& rc, const double* src, double* dst, int j)
{
    h->two.ring = rc.rows;
    h->two.lag = two_step_lag(h->g, rc.rows);
    h->two.epoch = ++h->two_epoch;
    h->two.cycles = make_wait_ctl(h->d_err).cycles;
    return launch_two_step_fx(src, dst, h->g, h->fx, h->two, rc.ctas_per_sm, j, h->d_fail, h->stream);
}

// Time every candidate in interleaved rounds (so that a drift of the clock
// or of the memory system during tuning does not favour one candidate) and
// keep each candidate's fastest round; the fastest candidate wins.
int tune(imex_lattice* h)
{
    std::vector<RowConfig> cands = row_candidates(h);
    RowConfig best{};  // classic
    if (!cands.empty()) {
        cands.insert(cands.begin(), RowConfig{});
        std::vector<float> fastest(cands.size(), 0.f);
        for (int round = 0; round < 4; ++round)
            for (size_t c = 0; c < cands.size(); ++c) {
                float ms = 0.f;
                const int reps = round == 0 ? 1 : 4;  // round 0 warms up
                int rc = c == 0 && use_fixed(h) ? time_fixed_run(h, reps, &ms) : time_shape(h, cands[c], reps, &ms);
                if (rc) return rc;
                if (round == 1 || ms < fastest[c]) fastest[c] = ms;
            }
        size_t b = 0;
        for (size_t c = 1; c < cands.size(); ++c)
            if (fastest[c] < fastest[b]) b = c;
        best = cands[b];
    }
    h->rows = best;
    std::lock_guard<std::mutex> guard(g_tune_lock);
    g_tune_cache[tune_key(h)] = best;
    return IMEX_OK;
}

// Pick the fused step's launch shape before its first use: a pinned shape,
// a cached result, the tuner, or - while the stream is being captured into
// a graph, where the tuner cannot synchronise - the first candidate.
int ensure_tuned(imex_lattice* h)
{
    if (h->shape_mode >= 0) return IMEX_OK;
    {
        std::lock_guard<std::mutex> guard(g_tune_lock);
        auto it = g_tune_cache.find(tune_key(h));
        if (it != g_tune_cache.end()) {
            h->rows = it->second;
            h->shape_mode = h->rows.stages > 1 ? 1 : 0;
            return IMEX_OK;
        }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    IMEX_CUDA(h, cudaStreamIsCapturing(h->stream, &cs), "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone) {
        std::vector<RowConfig> c = row_candidates(h);
        h->rows = c.empty() ? RowConfig{} : c.front();
        h->shape_mode = h->rows.stages > 1 ? 1 : 0;
        return IMEX_OK;
    }
    int rc = tune(h);
    if (rc) return rc;
    h->shape_mode = h->rows.stages > 1 ? 1 : 0;
    return IMEX_OK;
}

// One step-kernel launch in `mode` from buf[cur] into buf[cur] (collide) or
// buf[1 - cur] (fused / stream).
int launch_mode(imex_lattice* h, int mode)
{
    const double* src = dbuf(h, h->cur);
    double* dst = mode == kModeCollide ? dbuf(h, h->cur) : dbuf(h, 1 - h->cur);
    cudaError_t e;
    if (mode == kModeFused) {
        int rc = ensure_tuned(h);
        if (rc) return rc;
    }
    h->cf32.seed = (uint32_t)h->steps;  // stochastic rounding: a new stream of bits every step
    PhaseScope timed(h->prof, mode == kModeStream ? IMEX_PHASE_STREAM : IMEX_PHASE_COLLISION, h->stream);
    if (mode == kModeFused && h->rows.stages > 1)
        e = launch_fused_rows(h, src, dst, h->rows);
    else if (is_lowp(h))
        e = launch_step_lowp(h->precision, mode, src, dst, h->g, h->cf32, h->stream);
    else if (mode != kModeStream && use_fixed(h))
        e = launch_step_fx(mode, src, dst, h->g, h->fx, h->cf64, h->d_fallback, h->stream);
    else
        e = launch_step_f64(mode, src, dst, h->g, h->cf64, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "step kernel launch");
    ++h->launches;
    if (mode != kModeCollide) h->cur = 1 - h->cur;
    return IMEX_OK;
}

int check_ready(imex_lattice* h, const char* what)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": null handle");
    if (h->tag == kUninit) return fail(h, IMEX_ERR_STATE, std::string(what) + ": lattice not initialised");
    IMEX_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    return IMEX_OK;
}

// Make the device buffer hold the reference's f exactly (apply a pending
// streaming into the other buffer).
// A kernel's bounded wait ran out (see bulk.cuh): report it once.
int check_kernel_error(imex_lattice* h)
{
    unsigned v = 0;
    IMEX_CUDA(h, cudaMemcpyAsync(&v, h->d_err, sizeof v, cudaMemcpyDeviceToHost, h->stream), "cudaMemcpy");
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), "kernel status");
    if (v) {
        IMEX_CUDA(h, cudaMemsetAsync(h->d_err, 0, sizeof v, h->stream), "cudaMemset");
        return fail(h, IMEX_ERR_CUDA, "a kernel's asynchronous copy did not complete in time; its results are invalid");
    }
    return IMEX_OK;
}

// Device view of a pinned (page-locked) host buffer, or nullptr for any
// other pointer (pageable memory is copied through the driver instead).
double* host_device_view(double* p)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return static_cast<double*>(at.devicePointer);
}


}  // namespace

extern "C" {

const char* imex_version(void) { return "imexlbm-gb300 0.2"; }

int imex_test_set_fault(int kind, long long value)
{
    if (kind == IMEX_TEST_FAULT_NONE) {
        g_fault_kind.store(kind);
        g_fault_value.store(0);
        return IMEX_OK;
    }
    if (kind == IMEX_TEST_FAULT_STARVE_STAGE && (value < 1000 || value > bulk::kWaitCycles))
        return set_thread_error(IMEX_ERR_ARG, "imex_test_set_fault: the wait limit must be in [1000, 2^31] SM clocks");
    if (kind != IMEX_TEST_FAULT_STARVE_STAGE && kind != IMEX_TEST_FAULT_BATCH_TABLE)
        return set_thread_error(IMEX_ERR_ARG, "imex_test_set_fault: unknown fault");
    g_fault_value.store(value);
    g_fault_kind.store(kind);
    return IMEX_OK;
}

const char* imex_last_error(const imex_lattice* h) { return h ? h->err.c_str() : thread_error(); }

int imex_create(int nx, int ny, int nz, double tau, double rho0, double u0, int precision, imex_lattice** out)
{
    if (!out) return set_thread_error(IMEX_ERR_ARG, "imex_create: null output pointer");
    *out = nullptr;
    if (nx < 1 || ny < 1 || nz < 1) return set_thread_error(IMEX_ERR_ARG, "imex_create: lattice sizes must be >= 1");
    if ((long long)ny * nx > 2147483647LL || nx > 65535 || ny > 65535)
        return set_thread_error(IMEX_ERR_ARG, "imex_create: nx and ny must be <= 65535");
    if (!std::isfinite(tau) || !std::isfinite(rho0) || !std::isfinite(u0) || !(tau + 0.5 > 0.0))
        return set_thread_error(IMEX_ERR_ARG, "imex_create: tau, rho0, u0 must be finite with tau > -0.5");
    if (precision != IMEX_F64 && precision != IMEX_F32 && precision != IMEX_F16DEV)
        return set_thread_error(IMEX_ERR_ARG, "imex_create: precision must be IMEX_F64, IMEX_F32 or IMEX_F16DEV");

    imex_lattice* h = new (std::nothrow) imex_lattice();
    if (!h) return set_thread_error(IMEX_ERR_MEMORY, "imex_create: host allocation failed");
    h->g.nx = nx;
    h->g.ny = ny;
    h->g.nz = nz;
    h->ncells = (size_t)nx * ny * nz;
    h->g.plane = h->ncells;
    h->tau0 = tau;
    h->rho0 = rho0;
    h->u0 = u0;
    h->precision = precision;
    h->cf64 = make_collide_f64(tau);
    h->cf32 = make_collide_f32(tau);
    h->cf32.sr = precision == IMEX_F16DEV;  // float16 deviations: stochastic rounding by default
    h->fx_ok = make_fx_params(tau, rho0, &h->fx);

    auto bail = [&](int code) {
        imex_destroy(h);
        return code;
    };
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaGetDevice"));

    const size_t arr = (size_t)kQ * h->ncells * elem_size(precision);
    const size_t nparts = conserved_partials(h->g);
    // scratch: conserved partials, 5 reduced values, fallback counter, error
    // flag, fixed-point run flag
    const size_t scratch = nparts * 5 * sizeof(double) + 5 * sizeof(double) + 3 * sizeof(unsigned long long);
    const size_t need = 2 * arr + scratch;
    // Device memory comes from the device's stream-ordered pool: creating
    // and destroying lattices (a server does it per request) then neither
    // synchronises the device nor returns memory to the driver.  Memory the
    // pool holds but no lattice uses counts as free.
    cudaMemPool_t pool = nullptr;
    e = cudaDeviceGetDefaultMemPool(&pool, h->device);
    size_t free_b = 0, total_b = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMemGetInfo"));
    unsigned long long reserved = 0, used = 0;
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    const size_t avail = free_b + (reserved > used ? (size_t)(reserved - used) : 0);
    if (need > avail) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "imex_create: needs %.3f GB of device memory, %.3f GB free", need / 1e9,
                      avail / 1e9);
        return bail(set_thread_error(IMEX_ERR_MEMORY, msg));
    }
    e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaStreamCreate"));
    h->stream = h->own_stream;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) e = cudaMallocAsync(&h->buf[b], arr, h->stream);
    unsigned char* s = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&s, scratch, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(set_thread_error(IMEX_ERR_MEMORY, "imex_create: device allocation failed"));
    }
    h->scratch = s;
    h->d_partial = reinterpret_cast<double*>(s);
    h->d_out = h->d_partial + nparts * 5;
    h->d_fallback = reinterpret_cast<unsigned long long*>(h->d_out + 5);
    h->d_err = reinterpret_cast<unsigned*>(h->d_fallback + 1);
    h->d_fail = reinterpret_cast<int*>(h->d_fallback + 2);
    e = cudaMemsetAsync(h->d_fallback, 0, 3 * sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // usable from any stream from here on
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "imex_create"));
    h->bytes = need;
    *out = h;
    return IMEX_OK;
}

void imex_destroy(imex_lattice* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->own_stream) {
        // release after the handle's queued work, on whichever stream it is
        if (h->stream && h->stream != h->own_stream) {
            cudaEvent_t ev;
            if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
                cudaEventRecord(ev, h->stream);
                cudaStreamWaitEvent(h->own_stream, ev, 0);
                cudaEventDestroy(ev);
            }
        }
        for (void* p : h->buf)
            if (p) cudaFreeAsync(p, h->own_stream);
        if (h->scratch) cudaFreeAsync(h->scratch, h->own_stream);
        if (h->two_mem) cudaFreeAsync(h->two_mem, h->own_stream);
        cudaStreamDestroy(h->own_stream);
    }
    delete h;
}

int imex_initialize(imex_lattice* h) { return imex_initialize_phase(h, 0.0, 0.0, 0.0); }

int imex_initialize_phase(imex_lattice* h, double phx, double phy, double phz)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_initialize: null handle");
    if (!std::isfinite(phx) || !std::isfinite(phy) || !std::isfinite(phz))
        return fail(h, IMEX_ERR_ARG, "imex_initialize_phase: phases must be finite");
    const double phase[3] = {phx, phy, phz};
    IMEX_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    // Per-axis trigonometric tables, src/lbm.cpp:81-93:
    //   x = (double)(i - ghost + x_lo) / (double)glx * 2.0 * pi, pi = 3.1415926
    const int n[3] = {h->g.nx, h->g.ny, h->g.nz};
    const size_t tot = 3 * ((size_t)n[0] + n[1] + n[2]);
    std::vector<double> table(tot);
    double* host = table.data();
    size_t off = 0;
    size_t offs[3];
    for (int d = 0; d < 3; ++d) {
        offs[d] = off;
        for (int i = 0; i < n[d]; ++i) {
            const double xx = (double)i / (double)n[d] * 2.0 * 3.1415926 + phase[d];
            host[off++] = std::sin(xx);
            host[off++] = std::cos(xx);
            host[off++] = std::cos(2.0 * xx);
        }
    }
    double* dev = nullptr;
    cudaError_t e = cudaMallocAsync(&dev, tot * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dev, host, tot * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = is_lowp(h) ? launch_init_lowp(h->precision, h->buf[0], h->g, dev + offs[0], dev + offs[1], dev + offs[2], h->rho0,
                                       h->u0, h->stream)
                    : launch_init_f64(dbuf(h, 0), h->g, dev + offs[0], dev + offs[1], dev + offs[2], h->rho0, h->u0,
                                      h->stream);
    if (e == cudaSuccess) {
        ++h->launches;
        e = cudaFreeAsync(dev, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_initialize");
    h->cur = 0;
    h->tag = kExact;
    h->steps = 0;
    return IMEX_OK;
}

int imex_collision(imex_lattice* h)
{
    int rc = check_ready(h, "imex_collision");
    if (rc) return rc;
    if (h->tag == kExact) return launch_mode(h, kModeCollide);
    rc = launch_mode(h, kModeFused);
    if (rc) return rc;
    h->tag = kExact;
    return IMEX_OK;
}

int imex_streaming(imex_lattice* h)
{
    int rc = check_ready(h, "imex_streaming");
    if (rc) return rc;
    if (h->tag == kPendingStream) {
        rc = launch_mode(h, kModeStream);
        if (rc) return rc;
    }
    h->tag = kPendingStream;
    ++h->steps;
    return IMEX_OK;
}

}  // extern "C"

namespace {

// The reference's time step (Collision then Streaming), one at a time.
int step_each(imex_lattice* h, int nsteps)
{
    for (int s = 0; s < nsteps; ++s) {
        int rc = imex_collision(h);
        if (rc) return rc;
        rc = imex_streaming(h);
        if (rc) return rc;
    }
    return IMEX_OK;
}

// n >= 2 steps of the float64 fixed-point engine in the steady state as one
// run that holds the state as X between its launches (launch_step_fx_run):
// the same numbers as n fused steps of k_step_fx, 4% faster at 256^3.  A
// cell leaving the exact range stops the run at that step; the run is then
// redone from the last complete step by k_step_fx, whose native float64
// fallback handles such cells.  The run ends with a synchronisation (to read
// that flag), so it is not used while the stream is being captured.
int step_fixed_run(imex_lattice* h, int n)
{
    const int64_t steps0 = h->steps;
    // the launches of the run: first step and the buffer each reads
    std::vector<std::pair<int, int>> runs;
    const bool two = h->rows.stages == 1;  // two steps per launch where it can
    if (two) {
        int rc = ensure_two_step(h, h->rows.rows);
        if (rc) return rc;
    }
    IMEX_CUDA(h, cudaMemsetAsync(h->d_fail, 0x7f, sizeof(int), h->stream), "cudaMemset");
    for (int j = 1; j <= n;) {
        PhaseScope timed(h->prof, IMEX_PHASE_COLLISION, h->stream);
        runs.emplace_back(j, h->cur);
        // a pair holds fixed point in and out: not the run's first or last step
        const bool pair = two && j > 1 && j + 1 < n;
        cudaError_t e = pair ? launch_two(h, h->rows, dbuf(h, h->cur), dbuf(h, 1 - h->cur), j)
                             : launch_step_fx_run(dbuf(h, h->cur), dbuf(h, 1 - h->cur), h->g, h->fx, j, n, h->d_fail,
                                                  h->stream);
        IMEX_CUDA(h, e, "step kernel launch");
        ++h->launches;
        h->cur = 1 - h->cur;
        const int k = pair ? 2 : 1;
        h->steps += k;
        j += k;
    }
    int failed = 0;
    IMEX_CUDA(h, cudaMemcpyAsync(&failed, h->d_fail, sizeof failed, cudaMemcpyDeviceToHost, h->stream), "cudaMemcpy");
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), "fixed-point run");
    if (two) {
        int rc = check_kernel_error(h);  // a bounded wait of the two-step kernel ran out
        if (rc) return rc;
    }
    if (failed > n) {
        h->fx_backoff = 0;
        return IMEX_OK;
    }
    // A cell left the exact range: the next calls step one at a time (a
    // run would likely fail again and be redone), for 1, 2, 4 .. 64 calls
    // after successive failures, then a run is tried again.
    h->fx_backoff = h->fx_backoff ? std::min(64, 2 * h->fx_backoff) : 1;
    h->fx_skip = h->fx_backoff;
    // state after step failed - 1: the source buffer of the launch that
    // began with step `failed` (a two-step launch records its first step)
    ++h->fx_reruns;
    for (const auto& r : runs)
        if (r.first == failed) h->cur = r.second;
    h->steps = steps0 + failed - 1;
    if (failed > 1) IMEX_CUDA(h, launch_fx_to_f64(dbuf(h, h->cur), (size_t)kQ * h->ncells, h->stream), "conversion");
    return step_each(h, n - failed + 1);
}

bool capturing(imex_lattice* h)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

}  // namespace

extern "C" {

int imex_step(imex_lattice* h, int nsteps)
{
    if (nsteps < 0) return fail(h, IMEX_ERR_ARG, "imex_step: nsteps < 0");
    int rc = check_ready(h, "imex_step");
    if (rc) return rc;
    if (use_fixed(h) && nsteps >= 3) {
        // reach the steady state (buffer pending a streaming) and the
        // launch shape, then run the rest as one fixed-point run when the
        // shape is one thread per cell
        if (h->tag != kPendingStream) {
            rc = step_each(h, 1);
            if (rc) return rc;
            --nsteps;
        }
        rc = ensure_tuned(h);
        if (rc) return rc;
        if (h->rows.stages <= 1 && !capturing(h)) {  // one thread per cell (1: two steps per launch)
            if (h->fx_skip > 0) {  // a recent run failed: step one at a time
                --h->fx_skip;
                return step_each(h, nsteps);
            }
            return step_fixed_run(h, nsteps);
        }
    }
    return step_each(h, nsteps);
}

int imex_conserved(imex_lattice* h, double out[5])
{
    int rc = check_ready(h, "imex_conserved");
    if (rc) return rc;
    if (!out) return fail(h, IMEX_ERR_ARG, "imex_conserved: null output");
    const bool pull = h->tag == kPendingStream;
    int timed = h->prof.start(IMEX_PHASE_CONSERVED, h->stream);
    cudaError_t e =
        is_lowp(h) ? launch_conserved_lowp(h->precision, pull, h->buf[h->cur], h->g, h->d_partial, h->d_out, h->stream)
        : use_fixed(h) ? launch_conserved_fx(pull, dbuf(h, h->cur), h->g, h->fx, h->d_partial, h->d_out, h->stream)
                       : launch_conserved_f64(pull, dbuf(h, h->cur), h->g, h->d_partial, h->d_out, h->stream);
    h->prof.stop(timed, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "conserved kernel launch");
    h->launches += 2;
    double res[5];
    IMEX_CUDA(h, cudaMemcpyAsync(res, h->d_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "cudaMemcpy");
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), "imex_conserved");
    rc = check_kernel_error(h);
    if (rc) return rc;
    bool finite = true;
    for (int q = 0; q < 5; ++q) {
        out[q] = res[q];
        finite = finite && std::isfinite(out[q]);
    }
    if (!finite) return fail(h, IMEX_ERR_NONFINITE, "imex_conserved: non-finite diagnostics (the run diverged)");
    return IMEX_OK;
}

}  // extern "C"

namespace {

// Per-cell p (optional), u, v, w of the handle's current distributions into
// device arrays of ncells doubles each, on the handle's stream.
int macro_fields(imex_lattice* h, double* p, double* u, double* v, double* w)
{
    const bool pull = h->tag == kPendingStream;
    PhaseScope timed(h->prof, IMEX_PHASE_MACRO, h->stream);
    cudaError_t e = is_lowp(h) ? launch_macro_lowp(h->precision, pull, h->buf[h->cur], h->g, p, u, v, w, h->stream)
                            : launch_macro_f64(pull, dbuf(h, h->cur), h->g, p, u, v, w, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "macroscopic kernel launch");
    ++h->launches;
    return IMEX_OK;
}

}  // namespace

extern "C" {

int imex_macroscopic(imex_lattice* h, double* p, double* u, double* v, double* w)
{
    int rc = check_ready(h, "imex_macroscopic");
    if (rc) return rc;
    const size_t nb = h->ncells * sizeof(double);
    double* d = nullptr;
    IMEX_CUDA(h, cudaMallocAsync(&d, 4 * nb, h->stream), "cudaMallocAsync");
    rc = macro_fields(h, d, d + h->ncells, d + 2 * h->ncells, d + 3 * h->ncells);
    cudaError_t e = cudaSuccess;
    double* outs[4] = {p, u, v, w};
    for (int q = 0; q < 4 && rc == IMEX_OK && e == cudaSuccess; ++q)
        if (outs[q]) e = cudaMemcpyAsync(outs[q], d + q * h->ncells, nb, cudaMemcpyDeviceToHost, h->stream);
    cudaError_t e2 = cudaFreeAsync(d, h->stream);
    if (rc) return rc;
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "imex_macroscopic");
    return IMEX_OK;
}

int imex_velocity_max_diff(imex_lattice* a, imex_lattice* b, double out[2])
{
    int rc = check_ready(a, "imex_velocity_max_diff");
    if (rc) return rc;
    rc = check_ready(b, "imex_velocity_max_diff");
    if (rc) return rc;
    if (!out) return fail(a, IMEX_ERR_ARG, "imex_velocity_max_diff: null output");
    if (a->g.nx != b->g.nx || a->g.ny != b->g.ny || a->g.nz != b->g.nz || a->device != b->device)
        return fail(a, IMEX_ERR_ARG, "imex_velocity_max_diff: lattices differ in size or device");
    IMEX_CUDA(a, cudaStreamSynchronize(b->stream), "imex_velocity_max_diff");
    const size_t n = a->ncells;
    double* d = nullptr;
    IMEX_CUDA(a, cudaMallocAsync(&d, 6 * n * sizeof(double) + 2 * sizeof(unsigned long long), a->stream),
              "cudaMallocAsync");
    cudaStream_t keep = b->stream;
    b->stream = a->stream;  // run b's kernel on a's stream, after a's work
    rc = macro_fields(a, nullptr, d, d + n, d + 2 * n);
    if (!rc) rc = macro_fields(b, nullptr, d + 3 * n, d + 4 * n, d + 5 * n);
    b->stream = keep;
    unsigned long long* res = reinterpret_cast<unsigned long long*>(d + 6 * n);
    unsigned long long host[2] = {0, 0};
    cudaError_t e = rc ? cudaSuccess : launch_maxdiff3(d, d + 3 * n, n, res, a->stream);
    if (!rc && e == cudaSuccess) {
        ++a->launches;
        e = cudaMemcpyAsync(host, res, sizeof host, cudaMemcpyDeviceToHost, a->stream);
    }
    cudaError_t e2 = cudaFreeAsync(d, a->stream);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(a, e, "imex_velocity_max_diff");
    std::memcpy(&out[0], &host[0], 8);
    std::memcpy(&out[1], &host[1], 8);
    return IMEX_OK;
}

static int get_f_impl(imex_lattice* h, double* dst, size_t n, cudaMemcpyKind kind, const char* what)
{
    int rc = check_ready(h, what);
    if (rc) return rc;
    if (!dst || n != (size_t)kQ * h->ncells) return fail(h, IMEX_ERR_ARG, std::string(what) + ": buffer size must be 27*nx*ny*nz");
    if (is_lowp(h)) {
        // convert (pulling through a pending streaming) into a float64
        // buffer: the destination itself when the device can write it (a
        // device buffer, or pinned host memory through its device view)
        double* tmp = kind == cudaMemcpyDeviceToDevice ? dst : host_device_view(dst);
        const bool staged = tmp == nullptr;
        if (staged) IMEX_CUDA(h, cudaMallocAsync(&tmp, n * sizeof(double), h->stream), "cudaMallocAsync");
        cudaError_t e = launch_to_f64(h->precision, h->tag == kPendingStream, h->buf[h->cur], h->g, tmp, h->stream);
        if (e == cudaSuccess) ++h->launches;
        if (e == cudaSuccess && staged) e = cudaMemcpyAsync(dst, tmp, n * sizeof(double), kind, h->stream);
        if (staged) cudaFreeAsync(tmp, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, what);
        return IMEX_OK;
    }
    if (h->tag != kPendingStream) {
        IMEX_CUDA(h, cudaMemcpyAsync(dst, dbuf(h, h->cur), n * sizeof(double), kind, h->stream), what);
        IMEX_CUDA(h, cudaStreamSynchronize(h->stream), what);
        return IMEX_OK;
    }
    // A streaming is pending: one kernel pulls the buffer through S into
    // the destination - the caller's device buffer, or a pinned host
    // buffer through its device view (written over the chip-to-chip link,
    // no staging copy) - and otherwise into the spare buffer, which is
    // then copied out.  The handle stays pending either way, so the next
    // fused step (or fixed-point run) proceeds as if nothing was read.
    double* target = kind == cudaMemcpyDeviceToDevice ? dst : host_device_view(dst);
    double* out = target ? target : dbuf(h, 1 - h->cur);
    {
        PhaseScope timed(h->prof, IMEX_PHASE_STREAM, h->stream);
        IMEX_CUDA(h, launch_step_f64(kModeStream, dbuf(h, h->cur), out, h->g, h->cf64, h->stream), "stream kernel launch");
    }
    ++h->launches;
    if (!target) IMEX_CUDA(h, cudaMemcpyAsync(dst, out, n * sizeof(double), kind, h->stream), what);
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), what);
    return IMEX_OK;
}

static int set_f_impl(imex_lattice* h, const double* src, size_t n, cudaMemcpyKind kind, const char* what)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": null handle");
    if (!src || n != (size_t)kQ * h->ncells) return fail(h, IMEX_ERR_ARG, std::string(what) + ": buffer size must be 27*nx*ny*nz");
    IMEX_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    if (is_lowp(h)) {
        const double* dsrc = src;
        double* tmp = nullptr;
        cudaError_t e = cudaSuccess;
        if (kind != cudaMemcpyDeviceToDevice) {
            e = cudaMallocAsync(&tmp, n * sizeof(double), h->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, src, n * sizeof(double), kind, h->stream);
            dsrc = tmp;
        }
        if (e == cudaSuccess) e = launch_from_f64(h->precision, dsrc, h->buf[h->cur], h->g, h->stream);
        if (e == cudaSuccess) ++h->launches;
        if (tmp) cudaFreeAsync(tmp, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, what);
    } else {
        IMEX_CUDA(h, cudaMemcpyAsync(dbuf(h, h->cur), src, n * sizeof(double), kind, h->stream), what);
        IMEX_CUDA(h, cudaStreamSynchronize(h->stream), what);
    }
    h->tag = kExact;
    return IMEX_OK;
}

int imex_get_f(imex_lattice* h, double* host, size_t n) { return get_f_impl(h, host, n, cudaMemcpyDeviceToHost, "imex_get_f"); }
int imex_set_f(imex_lattice* h, const double* host, size_t n) { return set_f_impl(h, host, n, cudaMemcpyHostToDevice, "imex_set_f"); }
int imex_get_f_device(imex_lattice* h, double* dev, size_t n)
{
    return get_f_impl(h, dev, n, cudaMemcpyDeviceToDevice, "imex_get_f_device");
}
int imex_set_f_device(imex_lattice* h, const double* dev, size_t n)
{
    return set_f_impl(h, dev, n, cudaMemcpyDeviceToDevice, "imex_set_f_device");
}

int imex_set_engine(imex_lattice* h, int engine)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_set_engine: null handle");
    if (engine != IMEX_ENGINE_AUTO && engine != IMEX_ENGINE_NATIVE && engine != IMEX_ENGINE_FIXED)
        return fail(h, IMEX_ERR_ARG, "imex_set_engine: unknown engine");
    if (engine == IMEX_ENGINE_FIXED && (!h->fx_ok || is_lowp(h)))
        return fail(h, IMEX_ERR_ARG, "imex_set_engine: the fixed-point engine needs float64 storage and 0.75 <= rho0 <= 1.25");
    h->engine = engine;
    return IMEX_OK;
}

int imex_set_rounding(imex_lattice* h, int mode)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_set_rounding: null handle");
    if (mode != IMEX_ROUND_NEAREST && mode != IMEX_ROUND_STOCHASTIC)
        return fail(h, IMEX_ERR_ARG, "imex_set_rounding: unknown mode");
    if (mode == IMEX_ROUND_STOCHASTIC && h->precision != IMEX_F16DEV)
        return fail(h, IMEX_ERR_ARG, "imex_set_rounding: stochastic rounding applies to IMEX_F16DEV storage");
    const int sr = mode == IMEX_ROUND_STOCHASTIC;
    // a shape the autotuner chose for the other rounding mode is re-chosen
    if (sr != h->cf32.sr && !h->shape_pinned) h->shape_mode = -1;
    h->cf32.sr = sr;
    return IMEX_OK;
}

int imex_set_stream(imex_lattice* h, void* s)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_set_stream: null handle");
    h->stream = s ? static_cast<cudaStream_t>(s) : h->own_stream;
    return IMEX_OK;
}

int imex_profile_enable(imex_lattice* h, int on)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_profile_enable: null handle");
    IMEX_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    h->prof.enable(on != 0);
    return IMEX_OK;
}

int imex_profile_read(imex_lattice* h, imex_phase_stats out[IMEX_NPHASE], int reset)
{
    if (!h || !out) return set_thread_error(IMEX_ERR_ARG, "imex_profile_read: null argument");
    IMEX_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    h->prof.read(out, reset != 0);
    return IMEX_OK;
}

int imex_synchronize(imex_lattice* h)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_synchronize: null handle");
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), "imex_synchronize");
    return check_kernel_error(h);
}

int imex_set_launch(imex_lattice* h, int stages, int rows_per_stage, int ctas_per_sm)
{
    if (!h) return set_thread_error(IMEX_ERR_ARG, "imex_set_launch: null handle");
    if (stages < 0) {
        h->shape_mode = -1;
        h->shape_pinned = false;
        return IMEX_OK;
    }
    if (stages == 0 || stages == 1) {
        RowConfig rc{};
        rc.stages = stages;
        if (stages == 1) {  // rows_per_stage: ring depth; ctas_per_sm: resident CTAs
            rc.rows = rows_per_stage >= kTwoRingMin ? rows_per_stage : kTwoRingDefault;
            rc.ctas_per_sm = ctas_per_sm < 1 ? 5 : ctas_per_sm;
            if (!(use_fixed(h) && two_step_eligible(h->g, rc.rows)) || rc.ctas_per_sm > 6)
                return fail(h, IMEX_ERR_ARG, "imex_set_launch: two steps per launch (stages 1) needs the float64 "
                                             "fixed-point engine, nx >= 8, ny >= 4, a ring of 4..16 planes whose lag "
                                             "fits in the lattice and 1..6 CTAs per SM");
        }
        h->rows = rc;
        h->shape_mode = 0;
        h->shape_pinned = true;
        return IMEX_OK;
    }
    if (!rows_eligible_for(h))
        return fail(h, IMEX_ERR_ARG, "imex_set_launch: the row-staged kernel needs nz*element size a multiple of 16 "
                                     "bytes and a fixed-point or reduced-precision engine");
    const int B = rows_per_stage < 1 ? 1 : rows_per_stage;
    if (!is_lowp(h) && h->g.ny % B) return fail(h, IMEX_ERR_ARG, "imex_set_launch: rows_per_stage must divide ny");
    if (B > h->g.ny) return fail(h, IMEX_ERR_ARG, "imex_set_launch: rows_per_stage must not exceed ny");
    RowConfig rc;
    rc.stages = stages;
    rc.rows = B;
    rc.ctas_per_sm = ctas_per_sm < 1 ? 1 : ctas_per_sm;
    if (is_lowp(h)) {
        rc.dir_bytes = lowp_dir_bytes(h, B);
        rc.threads = rowslp::kThreads;
        if (!rc.dir_bytes || stages < 2 || stages > 16 || rowslp::smem_bytes(rc.dir_bytes, stages) > 227 * 1024)
            return fail(h, IMEX_ERR_ARG, "imex_set_launch: ring does not fit in shared memory (2 <= stages <= 16, "
                                         "rows_per_stage * nz * element size <= 4096 bytes)");
    } else {
        if (stages < 2 || stages > 16 || kRowBarrierBytes + (size_t)stages * B * stage_bytes(h) > 227 * 1024)
            return fail(h, IMEX_ERR_ARG, "imex_set_launch: ring does not fit in shared memory (2 <= stages <= 16)");
        rc.threads = h->g.nz >= 256 ? 256 : ((h->g.nz + 31) / 32) * 32;
    }
    h->rows = rc;
    h->shape_mode = 1;
    h->shape_pinned = true;
    return IMEX_OK;
}

int imex_get_launch(imex_lattice* h, int out[4])
{
    if (!h || !out) return set_thread_error(IMEX_ERR_ARG, "imex_get_launch: null argument");
    int rc = ensure_tuned(h);
    if (rc) return rc;
    out[0] = h->rows.stages;
    out[1] = h->rows.stages >= 1 ? h->rows.rows : 0;  // two steps per launch: the ring depth
    out[2] = h->rows.ctas_per_sm;
    out[3] = h->rows.stages > 1 ? h->rows.threads : kStepBlock;  // one thread per cell: blocks of kStepBlock
    return IMEX_OK;
}

int64_t imex_steps_done(const imex_lattice* h) { return h ? h->steps : -1; }
int64_t imex_kernel_launches(const imex_lattice* h) { return h ? h->launches : -1; }
size_t imex_device_bytes(const imex_lattice* h) { return h ? h->bytes : 0; }

int imex_fallback_cells(imex_lattice* h, int64_t* out, int reset)
{
    if (!h || !out) return set_thread_error(IMEX_ERR_ARG, "imex_fallback_cells: null argument");
    unsigned long long v = 0;
    IMEX_CUDA(h, cudaMemcpyAsync(&v, h->d_fallback, sizeof v, cudaMemcpyDeviceToHost, h->stream), "cudaMemcpy");
    IMEX_CUDA(h, cudaStreamSynchronize(h->stream), "imex_fallback_cells");
    if (reset) IMEX_CUDA(h, cudaMemsetAsync(h->d_fallback, 0, sizeof v, h->stream), "cudaMemset");
    *out = (int64_t)v;
    return IMEX_OK;
}

}  // extern "C"
