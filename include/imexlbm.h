/*
 * imexlbm.h - C ABI of the GB300-native IMEXLBM time step.
 *
 * One handle = one periodic D3Q27 lattice resident on one GPU.  The entry
 * points mirror the reference's single-rank call surface (struct LBM and
 * class System in Maccchiatooo/IMEXLBM); each declaration names the
 * reference interface it replaces as path:line within that project.
 *
 * Conventions
 *   - Every call returns an int status: IMEX_OK (0) or an IMEX_ERR_* code;
 *     imex_last_error(h) gives a one-line description for the handle.
 *   - The handle owns its device memory.  Calls on one handle are not
 *     thread-safe; separate handles may be driven from separate threads.
 *   - Work is queued on the handle's CUDA stream (default: a stream the
 *     handle creates).  Calls that return host data synchronise that stream.
 *   - Distribution arrays crossing the ABI are float64 in the reference's
 *     index order f[a][x][y][z] (z fastest), interior cells only: 27*nx*ny*nz
 *     values, a in the reference's direction order (src/lbm.cpp:20-30).
 */
#ifndef IMEXLBM_H
#define IMEXLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMEX_OK 0
#define IMEX_ERR_ARG 1       /* bad argument (null pointer, size, enum)            */
#define IMEX_ERR_CUDA 2      /* a CUDA runtime call failed                          */
#define IMEX_ERR_MEMORY 3    /* device allocation failed or over the HBM budget     */
#define IMEX_ERR_DECK 4      /* input deck missing or malformed                     */
#define IMEX_ERR_NONFINITE 5 /* diagnostics produced NaN or Inf                     */
#define IMEX_ERR_STATE 6     /* call out of sequence (e.g. step before initialize)  */
#define IMEX_ERR_IO 7        /* a file could not be opened, read or written         */

/* Storage precision of the distributions. */
#define IMEX_F64 0    /* float64 storage (the reference's own precision)        */
#define IMEX_F32 1    /* float32 storage, float32 collision                     */
#define IMEX_F16DEV 2 /* float16 storage of (f_a - w_a) * 2^12, float32 collision */

/* Rounding of float16-deviation storage (imex_set_rounding). */
#define IMEX_ROUND_NEAREST 0    /* round to nearest even                               */
#define IMEX_ROUND_STOCHASTIC 1 /* round up or down with probabilities (13-bit) that
                                   keep the expected stored value exact                 */

/* Arithmetic engine of the float64 collision. */
#define IMEX_ENGINE_AUTO 0   /* fastest engine that meets float64 parity            */
#define IMEX_ENGINE_NATIVE 1 /* native float64 FMA arithmetic                       */
#define IMEX_ENGINE_FIXED 2  /* exact 64-bit fixed-point arithmetic on the integer
                                pipes, rounded once to float64 per output          */

typedef struct imex_lattice imex_lattice;

/* Input deck: the nine numbers of input.in plus the derived quantities.
 * Field names and meanings follow class System (src/System.hpp:11-19). */
typedef struct imex_deck {
    double rho0, R, u0;
    int Re, Time, inter, sx, sy, sz;
    double cs2, cs, Ma, miu, tau;
} imex_deck;

/* ---------------------------------------------------------------- deck -- */

/* Parse deck text (nine whitespace-separated numbers; anything after the
 * ninth is ignored) and derive cs2, cs, Ma, miu, tau.
 * Replaces System::System() (src/System.cpp:11-29), which reads the same
 * fields with std::istream >> in the same order.  Where the reference aborts
 * on a missing or unreadable deck, this returns IMEX_ERR_DECK. */
int imex_deck_parse(const char *text, imex_deck *out);

/* Read and parse a deck file (System.cpp:16-24 reads "input.in" from CWD). */
int imex_deck_read(const char *path, imex_deck *out);

/* -------------------------------------------------------------- lattice -- */

/* Create a lattice handle and allocate its device arrays.
 * Replaces LBM::LBM(comm, sx, sy, sz, tau, rho0, u0) (src/lbm.hpp:179-183)
 * plus the allocations of LBM::Initialize (src/lbm.cpp:43-57).
 * precision: IMEX_F64 | IMEX_F32 | IMEX_F16DEV. */
int imex_create(int nx, int ny, int nz, double tau, double rho0, double u0,
                int precision, imex_lattice **out);

/* Free the handle and its device memory.  Safe on NULL. */
void imex_destroy(imex_lattice *h);

/* Taylor-Green initial field and equilibrium distributions.
 * Replaces LBM::Initialize() (src/lbm.cpp:38-111). */
int imex_initialize(imex_lattice *h);

/* Taylor-Green initial field with the coordinates shifted by a phase per
 * axis: x = i / nx * 2 pi + phx (and likewise y, z) in src/lbm.cpp:81-93.
 * imex_initialize is the zero-phase case.  Used to give the lattices of a
 * batch distinct flows; no counterpart in the reference. */
int imex_initialize_phase(imex_lattice *h, double phx, double phy, double phz);

/* BGK collision with relaxation rate 1/(tau0 + 0.5).
 * Replaces LBM::Collision() (src/lbm.cpp:131-166). */
int imex_collision(imex_lattice *h);

/* Periodic pull streaming.
 * Replaces LBM::Streaming() (src/lbm.cpp:168-207) including passf()
 * (src/mpi_view_transfer.cpp:451-456), whose one-rank halo is the periodic
 * image.  A Collision() followed by Streaming() runs as one fused
 * collide + pull-stream kernel; either call alone keeps its own meaning. */
int imex_streaming(imex_lattice *h);

/* Advance nsteps reference steps (Collision then Streaming, repeated).
 * Equivalent to the loop body of src/main.cpp:31-61 without reporting.
 * On the float64 fixed-point engine, nsteps >= 3 run as one run that keeps
 * the state in fixed point between its kernel launches (the same numbers,
 * bit for bit); such a call returns after the run has finished on the
 * device (it reads whether every cell stayed in the exact range), except
 * while the handle's stream is being captured. */
int imex_step(imex_lattice *h, int nsteps);

/* Global diagnostics of the current distributions: out = {mass, px, py, pz,
 * ke}.  Replaces LBM::Conserved() (src/lbm.cpp:266-306); synchronises.
 * Returns IMEX_ERR_NONFINITE (with out filled) if any value is NaN or Inf. */
int imex_conserved(imex_lattice *h, double out[5]);

/* Per-cell macroscopic fields p = sum f / 3 and (u, v, w) = sum f e, each
 * nx*ny*nz float64 on the host.  Replaces LBM::ComputeMacroscopic()
 * (src/lbm.cpp:213-240).  Any output pointer may be NULL. */
int imex_macroscopic(imex_lattice *h, double *p, double *u, double *v, double *w);

/* Largest velocity difference between two lattices of the same size on
 * the same GPU: out[0] = max over cells and components of |u_a - u_b|,
 * out[1] = max |u_b| (u = sum f e per cell, as in src/lbm.cpp:227-235).
 * Compares a reduced-precision run against a float64 run without moving
 * the fields to the host.  Synchronises both handles' streams. */
int imex_velocity_max_diff(imex_lattice *a, imex_lattice *b, double out[2]);

/* Per-phase device time of a lattice's kernels, for the per-phase profile
 * report of the reference's profiling build (src/profile.hpp:53-70,
 * src/profile.cpp:107-200).  While enabled, each kernel launch of the phase
 * is bracketed by CUDA events on the handle's stream - no synchronisation
 * is added to the step - and its device time is folded into calls, total,
 * min and max when the statistics are read.  Phases: */
#define IMEX_PHASE_COLLISION 0 /* fused step / collision kernels (P_COLLISION)   */
#define IMEX_PHASE_STREAM 1    /* streaming applied alone (P_STREAM_*)           */
#define IMEX_PHASE_MACRO 2     /* macroscopic fields, min/max, output (P_MACRO)  */
#define IMEX_PHASE_CONSERVED 3 /* conserved-quantity reduction                   */
#define IMEX_NPHASE 4
typedef struct imex_phase_stats {
    int64_t calls;
    double total_ms, min_ms, max_ms;
} imex_phase_stats;
int imex_profile_enable(imex_lattice *h, int on);
/* Read (and with reset != 0 clear) the statistics; waits for the timed
 * launches to finish. */
int imex_profile_read(imex_lattice *h, imex_phase_stats out[IMEX_NPHASE], int reset);

/* Extremes of the macroscopic fields: out = {umax, vmax, wmax, pmax, umin,
 * vmin, wmin, pmin} over all cells, with p = sum f / 3 and (u, v, w) =
 * sum f e as ComputeMacroscopic forms them.  The "minmax_uvwp" reduction of
 * LBM::MPIoutput (src/lbm.cpp:351-372), in its reducer order; NaN values
 * are skipped and an all-NaN field gives -DBL_MAX / DBL_MAX, the
 * reduction's identities.  One fused pass over f, no field arrays.
 * Synchronises. */
int imex_minmax_uvwp(imex_lattice *h, double out[8]);

/* Write the binary Tecplot file of LBM::MPIoutput(n) (src/lbm.cpp:307-598)
 * for this lattice: the 332-byte "#!TDV112" header with solution time n
 * and the field ranges, then seven float64 blocks x, y, z, u, v, w, p in
 * x-fastest order, node coordinates index / (extent - 1).  path NULL
 * writes "output<n>.plt" in the working directory, the reference's name.
 * Device staging: 32 bytes per cell for the duration of the call.
 * Returns IMEX_ERR_IO if the file cannot be written.  Synchronises. */
int imex_write_tecplot(imex_lattice *h, const char *path, int n);

/* Write the ASCII dump of LBM::Output(n) (src/lbm.cpp:606-636) for this
 * lattice: "variables=x,y,z,f", "zone I=nx,J=ny,K=nz", then one line
 * "x y z f" per cell, x fastest, with the rest population f(0) in fixed
 * notation with 8 decimals.  path NULL writes "output<n>0.dat" (the
 * reference's name on rank 0).  Returns IMEX_ERR_IO if the file cannot be
 * written.  Synchronises. */
int imex_write_output(imex_lattice *h, const char *path, int n);

/* Save the lattice's state - stored distributions in their storage
 * precision, the step count, whether a streaming is pending, the rounding
 * mode - to a file, and load it back into a lattice of the same size and
 * precision, which then continues bit for bit as the saved one would have
 * (stochastic rounding included).  tau, rho0 and u0 stay the loading
 * handle's own.  No reference counterpart: the reference has no restart
 * file.  Not while the lattice is a batch member.  Both synchronise. */
int imex_checkpoint_save(imex_lattice *h, const char *path);
int imex_checkpoint_load(imex_lattice *h, const char *path);

/* Copy the current distributions (reference order, float64) to the host
 * buffer of n = 27*nx*ny*nz values.  The reference exposes them as the
 * public member LBM::f (src/lbm.hpp:165).  A pending streaming is applied
 * on the way out by one kernel, without changing the handle's state; a
 * pinned (page-locked) host buffer is written by that kernel directly,
 * any other through a device staging copy.  Synchronises. */
int imex_get_f(imex_lattice *h, double *host, size_t n);

/* Overwrite the distributions from a host buffer of n = 27*nx*ny*nz
 * float64 values (reference order).  Marks the handle initialised. */
int imex_set_f(imex_lattice *h, const double *host, size_t n);

/* Same as imex_get_f / imex_set_f for a buffer already on this GPU. */
int imex_get_f_device(imex_lattice *h, double *dev, size_t n);
int imex_set_f_device(imex_lattice *h, const double *dev, size_t n);

/* Conserved diagnostics of distributions in a caller-owned device buffer,
 * without allocating anything.  No counterpart in the reference: it is for
 * callers that cannot call cudaMalloc - a host code whose device memory is
 * owned by its own pool allocator, or a latency-critical loop where
 * cudaMalloc's implicit device synchronisation is not acceptable.
 *   f_dev    27*nx*ny*nz float64 in the layout above, on the current device
 *   out_dev  5 float64 on the current device: {mass, px, py, pz, ke}, as
 *            imex_conserved computes them
 *   stream   cudaStream_t as void* (NULL: the legacy default stream); the
 *            call is asynchronous on it
 * Scratch: a file-scope static device array of 131072 partial sums (5 MiB),
 * which every GPU that loads this library holds until the process exits.
 * Lattices needing more partial sums than that (one per 128 z-cells of a
 * row, e.g. more than 256x256x256) are rejected with IMEX_ERR_ARG.  The
 * first call on each device looks the array's device address up
 * (cudaGetSymbolAddress) and keeps it for the process, so make that first
 * call before any stream capture; a cudaDeviceReset invalidates the kept
 * address, so do not call this entry point on a device after resetting it.
 * All calls share the array: calls that overlap on the GPU (on different
 * streams, or from different threads) race; serialise them.
 * Errors are reported through imex_last_error(NULL). */
int imex_conserved_noalloc(const double *f_dev, int nx, int ny, int nz, double *out_dev, void *stream);

/* Launch shape of the fused step.  stages = 0: one thread per cell pulling
 * straight from global memory.  stages = 1 (float64 fixed-point engine, nx
 * >= 8, ny >= 4; only when pinned, the automatic choice never takes it):
 * the same, with imex_step's runs taking two steps per launch - the first
 * step's values go to a ring of rows_per_stage + 2 x-planes in device
 * memory (rows_per_stage 4..16, below 4: 12) and the second step reads
 * them there, rows ordered across the GPU by tickets and per-row flags
 * (bounded waits), ctas_per_sm 1..6 resident CTAs (below 1: 5); the
 * numbers are the one-step form's, bit for bit, and it runs slower than
 * stages 0 on GB300 (10-30% at 128^3-256^3, more on small lattices).
 * imex_get_launch reports the ring depth as rows_per_stage.
 * stages >= 2: the row-staged kernel - each
 * CTA keeps a ring of `stages` work items in shared memory, an item being
 * rows_per_stage consecutive y-rows (dividing ny for float64; for reduced
 * precision the last item of a plane takes the rows left) whose 27 source row runs
 * arrive by asynchronous bulk copies - with ctas_per_sm resident CTAs per
 * SM; it needs nz * element size a multiple of 16 bytes and the fixed-point
 * or a reduced-precision engine.  stages < 0: back to automatic.  By
 * default the first fused step of a handle times every eligible shape on
 * the handle's own lattice (without changing its state) and keeps the
 * fastest, cached per lattice shape for the process; while the handle's
 * stream is being captured into a CUDA graph it takes the first eligible
 * shape instead.  No counterpart in the reference (Kokkos picks its own
 * tiles, src/lbm.cpp:135-139). */
int imex_set_launch(imex_lattice *h, int stages, int rows_per_stage, int ctas_per_sm);

/* The shape in use: out = {stages, rows_per_stage, ctas_per_sm, threads per
 * CTA}; runs the autotuner first if no shape has been chosen yet. */
int imex_get_launch(imex_lattice *h, int out[4]);

/* Select the float64 arithmetic engine (IMEX_ENGINE_*).  Default AUTO. */
int imex_set_engine(imex_lattice *h, int engine);

/* Rounding mode of IMEX_F16DEV storage (default IMEX_ROUND_STOCHASTIC).  At
 * omega close to 2 (high Reynolds number) the non-equilibrium part of each
 * population is far below half a float16 step of f - w, so rounding to
 * nearest erases it deterministically and biases the viscous decay (512^3,
 * Re 1600: kinetic energy off by 9e-9 per step); stochastic rounding keeps
 * it in expectation (1.3e-8 after 1000 steps).  Both modes keep each cell's
 * momentum: the momentum of the other populations' rounding errors is moved
 * into the eight corner populations before they are rounded.  The random
 * bits come from a hash of (cell, step), so runs are reproducible and
 * identical across kernels and batches. */
int imex_set_rounding(imex_lattice *h, int mode);

/* Queue the handle's work on an existing CUDA stream (cudaStream_t passed as
 * void*; NULL restores the handle's own stream). */
int imex_set_stream(imex_lattice *h, void *cuda_stream);

/* Wait for the handle's queued work (Kokkos::fence() in the reference). */
int imex_synchronize(imex_lattice *h);

/* Reference steps completed since initialisation. */
int64_t imex_steps_done(const imex_lattice *h);

/* Kernel launches queued by this handle since creation (all kernels). */
int64_t imex_kernel_launches(const imex_lattice *h);

/* Cells whose float64 collision left the fixed-point engine's exact range
 * and ran through the native float64 path instead, summed over all steps
 * since the last reset; 0 for other engines.  Synchronises. */
int imex_fallback_cells(imex_lattice *h, int64_t *out, int reset);

/* Device bytes held by the handle. */
size_t imex_device_bytes(const imex_lattice *h);

/* Last error message of the handle (or of the calling thread when h is
 * NULL, for errors raised before a handle exists).  Never NULL. */
const char *imex_last_error(const imex_lattice *h);

/* ---------------------------------------------------------------- batch -- */

/* Many float32 / float16-deviation lattices of any sizes, advanced together
 * by one persistent kernel launch per step over a packed cell index (no
 * counterpart in the reference, which runs one lattice per process).  The
 * batch holds handles created by imex_create; each member keeps its own
 * buffers, state, diagnostics (imex_conserved, imex_get_f ...) and
 * results identical bit for bit to stepping it alone.  Steps run on the
 * batch's own stream in CUDA graphs of K launches (imex_batch_set_graph);
 * the members' streams are ordered before and after each imex_batch_step.
 * Calls on one batch are not thread-safe. */
typedef struct imex_batch imex_batch;

/* Create an empty batch for up to max_members (<= 2048) lattices. */
int imex_batch_create(int max_members, imex_batch **out);
void imex_batch_destroy(imex_batch *b);

/* Add an initialised float32 / float16-deviation lattice (fewer than 2^32
 * cells).  max_steps >= 0 stops the member once imex_steps_done reaches it
 * (its later imex_batch_step calls skip it); -1 for no limit. */
int imex_batch_add(imex_batch *b, imex_lattice *h, int64_t max_steps);
int imex_batch_remove(imex_batch *b, imex_lattice *h);
int imex_batch_size(const imex_batch *b);

/* Advance every member nsteps reference steps (Collision then Streaming,
 * as imex_step), or up to its limit.  The first call times the launch
 * shapes (threads per CTA, cells per thread, CTAs per SM) on the batch
 * itself, without changing any member's state, and keeps the fastest. */
int imex_batch_step(imex_batch *b, int nsteps);
int imex_batch_synchronize(imex_batch *b);

/* Pin the launch shape of the one-thread-per-cell kernel: a persistent
 * grid (threads 128|256, cells_per_thread 1|2|4, ctas_per_sm * threads <=
 * 2048; CTAs beyond those that can be resident are not launched), or
 * cells_per_thread 0 with threads 128 - one CTA per 128-cell row segment of
 * every member, the one-lattice kernel's grid over the whole batch (its
 * CUDA graph is captured again when the members' segment count changes).
 * threads = 0 retunes. */
int imex_batch_set_launch(imex_batch *b, int threads, int cells_per_thread, int ctas_per_sm);
int imex_batch_get_launch(imex_batch *b, int out[3]);

/* Launch shape of the row-staged batch kernel, which takes the members
 * whose z-rows are a multiple of 16 bytes (nz * element size) and at most
 * dir_kb KiB: ring depth `stages`, `dir_kb` KiB per direction in a stage
 * (1, 2 or 4; a member's work item is the largest block of y-rows that
 * fits), resident CTAs per SM, and whether float32 members join it
 * (float32_members != 0) or stay in the cell kernel.  stages 0 autotunes
 * (default); -1 turns the row kernel off, so every member runs in the cell
 * kernel.  imex_batch_get_row_launch gives {stages, dir_kb, ctas_per_sm,
 * float32_members} (stages -1 when the tuner found the cell kernel
 * faster). */
int imex_batch_set_row_launch(imex_batch *b, int stages, int dir_kb, int ctas_per_sm, int float32_members);
int imex_batch_get_row_launch(imex_batch *b, int out[4]);

/* Steps per captured CUDA graph (default 16; 0 launches each step
 * directly). */
int imex_batch_set_graph(imex_batch *b, int steps_per_graph);

/* Kernel launches issued by the batch (one per batched step). */
int64_t imex_batch_kernel_launches(const imex_batch *b);
const char *imex_batch_last_error(const imex_batch *b);

/* --------------------------------------------------------------- server -- */

/* A request server with continuous batching (no counterpart in the
 * reference).  Callers submit Taylor-Green solves from any thread; a server
 * thread admits them in arrival order while a slot is free and their device
 * memory fits the budget, advances all admitted requests together in one
 * batched launch per step (CUDA graphs of steps_per_tick steps), and retires
 * each at its step count, between ticks, publishing its diagnostics.  New
 * requests join while others run; every result is bit-identical to running
 * the request alone. */
typedef struct imex_server imex_server;

typedef struct imex_request {
    int nx, ny, nz;       /* lattice size */
    int precision;        /* IMEX_F32 or IMEX_F16DEV */
    int rounding;         /* IMEX_ROUND_* (IMEX_F16DEV storage) */
    int pad;
    double tau, rho0, u0; /* as imex_create */
    double phase[3];      /* as imex_initialize_phase */
    int64_t steps;        /* step count to reach (from 0, or from the resumed state) */
    int64_t tag;          /* caller's tag, returned in the result */
    char resume_path[256]; /* "" or a checkpoint (imex_checkpoint_save) to start
                              from instead of the Taylor-Green field: pause and
                              resume of a served solve */
    char save_path[256];   /* "" or a file the final state is saved to
                              (imex_checkpoint_save) before the result is published */
} imex_request;

typedef struct imex_result {
    int64_t id, tag;
    int status;           /* IMEX_OK, or the error that stopped the request */
    int pad;
    double conserved[5];  /* mass, px, py, pz, ke after `steps` (imex_conserved) */
    int64_t steps;        /* steps run */
    int64_t cells;
    double t_submit, t_admit, t_done; /* seconds on the server clock */
} imex_result;

typedef struct imex_server_stats {
    int64_t queued, active, completed, bytes_in_use;
    int64_t cell_updates; /* lattice-cell updates done by the batch */
    int64_t ticks;
    double busy_seconds;  /* wall time inside ticks */
    double now;           /* server clock */
    int64_t failed;       /* 1 if the server thread stopped on an error */
} imex_server_stats;

/* Start a server on the current device with a device-memory budget for the
 * admitted requests' distributions, at most max_active (<= 2048) requests
 * in flight, and steps_per_tick steps per batched tick. */
int imex_server_create(size_t budget_bytes, int max_active, int steps_per_tick, imex_server **out);

/* Queue a request (thread-safe); *id identifies its result. */
int imex_server_submit(imex_server *s, const imex_request *req, int64_t *id);

/* Move up to max finished results into out (thread-safe, non-blocking);
 * *n receives how many. */
int imex_server_poll(imex_server *s, imex_result *out, int max, int *n);

int imex_server_get_stats(imex_server *s, imex_server_stats *out);

/* Seconds since the server started (the clock of the results' times). */
double imex_server_now(const imex_server *s);

/* Admission order: IMEX_POLICY_ARRIVAL (default, first come first served;
 * the head waits for memory, no overtaking) or IMEX_POLICY_LEAST_WORK (the
 * queued request with the fewest cells x steps first: a shorter median
 * time-to-result under overload; large requests wait until the queue
 * drains). */
#define IMEX_POLICY_ARRIVAL 0
#define IMEX_POLICY_LEAST_WORK 1
int imex_server_set_policy(imex_server *s, int policy);

/* Stop the server thread; requests still queued or running are dropped. */
void imex_server_destroy(imex_server *s);

/* -------------------------------------------------------- decomposition -- */

/* Spatial decomposition of one lattice into blocks, the reference's
 * multi-rank layout (src/mpi_view_transfer.cpp), with the halo pruned to
 * the directions that cross each channel.  The plan calls below are host
 * arithmetic (no GPU); a multi-rank host code can exchange the messages
 * they describe over its own transport. */

/* One rank's block: rank = coord[0] + rx*coord[2] + rx*rz*coord[1]
 * (src/mpi_view_transfer.cpp:97-99), cells lo .. lo+len-1 per axis
 * (setup_Local's block distribution, :163-195). */
typedef struct imex_block {
    int rank;
    int coord[3]; /* px, py, pz */
    int lo[3];    /* first global cell per axis */
    int len[3];   /* cells per axis */
} imex_block;

/* One of a rank's 26 halo channels, in the reference's order (faces left,
 * right, down, up, front, back; 12 edges; 8 corners;
 * src/mpi_view_transfer.cpp:101-161).  The rank sends its boundary box on
 * side `offset` to send_to and receives the box of ghost cells on side
 * -offset from recv_from.  Boxes are in padded block coordinates: 1..len
 * interior, 0 and len+1 the one-cell ghost shell.  The message carries only
 * the directions e_a that cross the channel (e_a equal to offset on its
 * non-zero axes): 9 for a face, 3 for an edge, 1 for a corner, in
 * reference order; ndir * ext[0] * ext[1] * ext[2] values. */
typedef struct imex_halo_msg {
    int channel;
    int offset[3];
    int send_to, recv_from;
    int send_lo[3], recv_lo[3], ext[3];
    int ndir;
    int dirs[9]; /* -1 past ndir */
} imex_halo_msg;

/* The rank grid {rx, ry, rz} of setup_Cartesian (src/mpi_view_transfer.cpp:
 * 53-95): among the factorisations of nranks in ascending (rx, ry) order,
 * the first whose integer block extents have the least spread.  Refuses
 * grids with more ranks than cells along an axis. */
int imex_decomp_grid(int nranks, int nx, int ny, int nz, int grid[3]);
int imex_decomp_block(int nranks, int nx, int ny, int nz, int rank, imex_block *out);
int imex_decomp_halo(int nranks, int nx, int ny, int nz, int rank, int channel, imex_halo_msg *out);

/* A lattice decomposed into nranks blocks held on the current GPU, stepped
 * as the reference's ranks step theirs (no counterpart as one object: the
 * reference runs one block per MPI rank).  Each block keeps float64
 * distributions in a padded box with a one-cell ghost shell; a step is one
 * fused pull + collision launch over every block (the fixed-point engine's
 * arithmetic, so 0.75 <= rho0 <= 1.25; runs of steps in fixed point, as
 * imex_step's) that also stores each boundary cell's outgoing values - the
 * pruned directions of the messages above - into the ghost shells of the
 * blocks they stream into: the halo exchange as the producer's stores.
 * Every f equals the undivided lattice's bit for bit; the conserved sums are
 * the blocks' sums added in rank order. */
typedef struct imex_domain imex_domain;
typedef struct imex_domain_stats {
    int nranks;
    int grid[3];
    int64_t steps, launches;
    int64_t halo_values_per_step; /* values the halo exchange moves per step */
    int64_t device_bytes;
} imex_domain_stats;

int imex_domain_create(int nx, int ny, int nz, int nranks, double tau, double rho0, double u0, imex_domain **out);
void imex_domain_destroy(imex_domain *d);
/* Taylor-Green initial field of each block at its global coordinates
 * (LBM::Initialize on every rank, src/lbm.cpp:38-111). */
int imex_domain_initialize(imex_domain *d);
/* nsteps reference steps (Collision then Streaming) of every block. */
int imex_domain_step(imex_domain *d, int nsteps);
/* out = {mass, px, py, pz, ke}: each block's sums, added in rank order
 * (LBM::Conserved's MPI_Allreduce, src/lbm.cpp:266-306).  Synchronises. */
int imex_domain_conserved(imex_domain *d, double out[5]);
/* The same per block: out[5 * rank + q]. */
int imex_domain_conserved_blocks(imex_domain *d, double *out);
/* The whole lattice's f (reference order, n = 27*nx*ny*nz) gathered from
 * the blocks.  Synchronises. */
int imex_domain_get_f(imex_domain *d, double *host, size_t n);
int imex_domain_info(const imex_domain *d, imex_domain_stats *out);
int imex_domain_fallback_cells(imex_domain *d, int64_t *out);
int imex_domain_synchronize(imex_domain *d);
const char *imex_domain_last_error(const imex_domain *d);

/* Library version string. */
const char *imex_version(void);

/* ----------------------------------------------------------- test hooks -- */

/* Make the device-side error paths fire, for tests; no counterpart in the
 * reference, whose failures abort (src/System.cpp:17-21).  The setting is
 * process-wide and read at every launch of the row-staged kernels;
 * IMEX_TEST_FAULT_NONE (the default) restores normal operation.  Neither
 * fault faults or hangs the GPU: every wait involved is bounded.
 *   IMEX_TEST_FAULT_STARVE_STAGE  CTA 0 of every row-staged launch
 *       (imex_set_launch stages >= 2, the batch row kernel) arms the first
 *       stage of its ring without issuing that stage's copies, and every
 *       bounded wait gives up after `value` SM clocks (1000 .. 2^31) instead
 *       of 2^31.  The CTA's first wait runs out, it records the failure,
 *       waits (bounded) for the copies it has in flight and returns; the next
 *       synchronising call (imex_conserved, imex_synchronize,
 *       imex_batch_synchronize) returns IMEX_ERR_CUDA.
 *   IMEX_TEST_FAULT_BATCH_TABLE   the batch row kernel is launched with a
 *       member-table capacity one below its member count, so it refuses the
 *       table; imex_batch_synchronize returns IMEX_ERR_CUDA.
 * The results of the steps run under a fault are invalid. */
#define IMEX_TEST_FAULT_NONE 0
#define IMEX_TEST_FAULT_STARVE_STAGE 1
#define IMEX_TEST_FAULT_BATCH_TABLE 2
int imex_test_set_fault(int kind, long long value);

#ifdef __cplusplus
}
#endif
#endif /* IMEXLBM_H */
