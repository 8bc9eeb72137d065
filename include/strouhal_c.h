/*
 * strouhal_c.h — C ABI of the GB300-native D3Q19 lattice-Boltzmann step.
 *
 * Drop-in boundary for the solver API of the reference's StrouhalCore
 * (Sources/StrouhalCore/Sim.swift). Every entry point names the Swift member
 * it replaces. Conventions:
 *   - every call returns an int status (STRO_OK = 0); on failure the text of
 *     the error is available from stro_last_error() (thread-local);
 *   - the library owns all device memory; caller arrays are copied in/out;
 *   - calls on one handle are synchronous and a handle must not be used from
 *     two threads at once (Simulation is not thread-safe either);
 *   - preconditions the reference enforces with a trap (odd step count on a
 *     probe) return STRO_ERR_STATE instead;
 *   - cell index n = (z * ny + y) * nx + x; DDF state is 19 planes of N values
 *     ("shifted" f_i - w_i), plane i at offset i * N, FP32 or IEEE binary16.
 */
#ifndef STROUHAL_C_H
#define STROUHAL_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STRO_ABI_VERSION 1

/* Status codes. */
enum {
    STRO_OK = 0,
    STRO_ERR_INVALID = 1,   /* bad argument or size */
    STRO_ERR_NO_DEVICE = 2, /* no CUDA device (Sim.swift:67-71 StrouhalError.noDevice) */
    STRO_ERR_CUDA = 3,      /* CUDA runtime error (Sim.swift:328-330 command buffer failure) */
    STRO_ERR_OOM = 4,       /* device allocation failed (Sim.swift:221) */
    STRO_ERR_STATE = 5,     /* precondition: e.g. probe after an odd step count (Sim.swift:335,360) */
    STRO_ERR_TIMEOUT = 6    /* a bounded device-side wait gave up */
};

/* Precision, Sim.swift:5-8: FP32 arithmetic over FP32 or FP16 ("fp16s") DDF storage. */
enum { STRO_FP32 = 0, STRO_FP16S = 1 };

/* Cell, Sim.swift:46-52 (flag values as Kernels.metal:65-69). */
enum { STRO_FLUID = 0, STRO_SOLID = 1, STRO_LID = 2, STRO_INFLOW = 3, STRO_OUTFLOW = 4 };

typedef struct stro_ctx stro_ctx;
typedef struct stro_sim stro_sim;

/* Arguments of Simulation.init (Sim.swift:195-200). omega_minus == omega is SRT. */
typedef struct stro_sim_desc {
    int32_t precision;     /* STRO_FP32 or STRO_FP16S */
    int32_t nx, ny, nz;
    float omega;           /* omega+ = 1/tau */
    float omega_minus;     /* omega- (set equal to omega for SRT) */
    float lid[3];          /* lid wall velocity target */
    float uin;             /* inflow peak (parabolic) or uniform target */
    int32_t ramp_steps;    /* cosine ramp length; 0 = none (Sim.swift:258-266) */
    float force[3];        /* uniform Guo body force density */
    float c_smago;         /* Smagorinsky Cs^2 (not Cs); 0 = LES off */
    int32_t wants_forces;  /* enable probe_force (Sim.swift:199,219) */
} stro_sim_desc;

/* Last error text of the calling thread ("" if none). */
const char* stro_last_error(void);
int stro_abi_version(void);

/* ---- context: GPU (Sim.swift:60-78) ------------------------------------ */
int stro_ctx_create(int device, stro_ctx** out);
int stro_ctx_destroy(stro_ctx* ctx);
/* Device name and SM count of the context's GPU. */
int stro_ctx_info(stro_ctx* ctx, char* name, size_t name_len, int* sm_count);

/* ---- simulation: Simulation (Sim.swift:153-459) ---------------------------- */
/* Simulation.init (Sim.swift:195-256). flags: N cell codes (STRO_*) in cell
 * order, replacing the Swift flags(x,y,z) closure; NULL = all fluid. The
 * state starts at rest (all shifted DDFs zero, Sim.swift:225). */
int stro_sim_create(stro_ctx* ctx, const stro_sim_desc* desc, const uint8_t* flags,
                    stro_sim** out);
int stro_sim_destroy(stro_sim* sim);

/* Mutable properties, Sim.swift:164-172. */
int stro_sim_set_omega(stro_sim* sim, float omega, float omega_minus);
int stro_sim_set_lid(stro_sim* sim, const float lid[3]);
int stro_sim_set_uin(stro_sim* sim, float uin);
int stro_sim_set_ramp_steps(stro_sim* sim, int32_t ramp_steps);
int stro_sim_set_force(stro_sim* sim, const float force[3]);
int stro_sim_set_c_smago(stro_sim* sim, float c_smago);
int stro_sim_set_inflow_uniform(stro_sim* sim, int inflow_uniform);
/* sponge = (x0, width, tau); enabled = 0 removes it (Sim.swift:172,277-279). */
int stro_sim_set_sponge(stro_sim* sim, int enabled, float x0, float width, float tau);

/* Simulation.setSolidFractions (Sim.swift:413-421): N floats, Noble-Torczynski eps. */
int stro_sim_set_solid_fractions(stro_sim* sim, const float* eps);
/* Extension with no reference counterpart: per-cell Guo force field added to
 * the uniform force, 3 planes of N floats (fx plane, fy plane, fz plane).
 * NULL removes it. */
int stro_sim_set_force_field(stro_sim* sim, const float* fxyz);

/* Simulation.initField (Sim.swift:424-439, Kernels.metal:393-453):
 * mode 0 rest, 1 2-D Taylor-Green, 2 3-D Taylor-Green; tau = 1/omega. */
int stro_sim_init_field(stro_sim* sim, uint32_t mode, float amplitude);

/* Raw state access, replacing direct writes/reads of Simulation.fBuf
 * (Sim.swift:159; used by Cases.swift:92-98). bytes must be 19*N*elem_size. */
int stro_sim_upload_state(stro_sim* sim, const void* host, size_t bytes);
int stro_sim_download_state(stro_sim* sim, void* host, size_t bytes);
int stro_sim_state_bytes(stro_sim* sim, size_t* bytes);

/* Simulation.run(steps:) (Sim.swift:288-331): advances the lattice, returns
 * when the GPU has finished. */
int stro_sim_run(stro_sim* sim, int64_t steps);
/* stepsDone (Sim.swift:176) and gpuSeconds (Sim.swift:178). */
int stro_sim_steps_done(stro_sim* sim, int64_t* steps);
int stro_sim_set_steps_done(stro_sim* sim, int64_t steps);
int stro_sim_gpu_seconds(stro_sim* sim, double* seconds);

/* Simulation.probeMoments (Sim.swift:334-353): N x (ux, uy, uz, rho) float,
 * velocity with the Guo half-force shift. Even step count only. */
int stro_sim_moments(stro_sim* sim, float* out4);
/* Simulation.probeForce(xRange:yRange:) (Sim.swift:359-372): runs 2 steps with
 * momentum exchange on the odd one and sums the per-cell force over
 * x in [x0,x1], y in [y0,y1] (inclusive), all z, in FP64 on the GPU in a fixed
 * order. Needs wants_forces and an even step count. */
int stro_sim_probe_force(stro_sim* sim, int32_t x0, int32_t x1, int32_t y0, int32_t y1,
                         double out[3]);
/* Sum over cells of |u|^2 (|u|^2 in FP32 as the host loop of
 * Cases.swift:1240-1243 forms it, summed in FP64 on the GPU). Even steps only. */
int stro_sim_kinetic_energy(stro_sim* sim, double* sum_u2);
/* Extension: sum over fluid cells of the local viscous dissipation rate
 * 2 nu S:S, with S = -(3 omega / (2 rho)) Pi_neq (lattice units, FP64 sum).
 * Even steps only. */
int stro_sim_dissipation(stro_sim* sim, double* sum_eps);
/* Extension: both sums from one reduction over the state (the values
 * stro_sim_kinetic_energy and stro_sim_dissipation return): out[0] = sum
 * |u|^2, out[1] = sum 2 nu S:S. Even steps only. */
int stro_sim_observables(stro_sim* sim, double out[2]);
/* Simulation.stateDigest (Sim.swift:441-444): SHA-256 of the raw state bytes,
 * 64 lowercase hex chars + NUL. */
int stro_sim_digest(stro_sim* sim, char hex[65]);
/* Ladder.measure (Ladder.swift:54-72) in one submission: `transient` steps
 * (rounded down to even), then chunks of max(2, stride - 2) (rounded down to
 * even) steps each followed by the two-step force probe over the box, until
 * sample_steps steps are taken. Each probe's FP64 box force is reduced into
 * a device buffer; the samples come back once, at the end: forces[3 k + d]
 * for sample k, steps_at[k] (optional) the step count after its probe. The
 * number of samples is returned in *samples; a capacity below it fails with
 * *samples set. Requires wants_forces and an even step count. */
int stro_sim_run_sampled(stro_sim* sim, int64_t transient, int64_t sample_steps, int64_t stride,
                         int32_t x0, int32_t x1, int32_t y0, int32_t y1, double* forces,
                         int64_t capacity, int64_t* samples, int64_t* steps_at);
/* The |u| colormap of slice z (colorize, Kernels.metal:465-500) into a
 * caller array of nx*ny RGBA binary16 texels (uint16 bit patterns), row y
 * written at ny-1-y as the reference's texture write. The velocity is formed
 * from the slice's DDFs as Simulation.probeMoments forms it (even step counts
 * only). Headless: no window, swapchain or graphics API. seconds (optional):
 * device time of the render kernel. */
int stro_sim_render_slice(stro_sim* sim, int32_t z, float uref, uint16_t* rgba, double* seconds);
/* Simulation.massSum (Sim.swift:447-458): sum of all 19*N slots in FP64. */
int stro_sim_mass(stro_sim* sim, double* total);
/* 1 if every DDF is finite, else 0 (failure detection, Cases.swift:1250-1252). */
int stro_sim_check_finite(stro_sim* sim, int* all_finite);

/* Launch shape of the step kernels: bx*by threads (a multiple of 32, at most
 * 256) per block over an x-y tile. Results do not depend on it. */
int stro_sim_set_block(stro_sim* sim, int32_t bx, int32_t by);
int stro_sim_get_block(stro_sim* sim, int32_t* bx, int32_t* by);
/* Kernel variant: 0 = one cell per thread (all lattices); 1 = FP16 storage,
 * two x-adjacent cells per thread with half2 accesses (periodic lattices,
 * nx a multiple of 64); 2 = row staging: tiles of whole rows move through
 * shared memory by bulk loads ahead of the compute and bulk stores after it
 * (periodic lattices, nx*element size a multiple of 16, ny a multiple of the
 * rows per tile); 3 = one cell per thread with registers capped at 64 for
 * more warps in flight (periodic lattices, blocks of at most 128 threads);
 * 4 / 5 = FP16 storage, 4 / 8 x-adjacent cells per thread with 8- / 16-byte
 * loads (periodic lattices, nx a multiple of 128 / 256; launch shape from
 * stro_sim_set_block: bx a multiple of 32 dividing nx/4 or nx/8, by dividing ny).
 * A lattice a variant does not apply to runs variant 0.
 * Results are identical for every variant. */
int stro_sim_set_variant(stro_sim* sim, int32_t variant);
int stro_sim_get_variant(stro_sim* sim, int32_t* variant);
/* Arithmetic of the step. STRO_ARITH_REFERENCE (default) evaluates the
 * reference's collision expressions as written (Kernels.metal:105-228), equal
 * in value to the reference kernel in FP32. STRO_ARITH_FUSED evaluates the
 * same collision in an algebraically equal form with fused multiply-adds,
 * pair sums for the moments and shared weight products: about a quarter
 * fewer instructions per cell, results differ from the reference
 * arithmetic in the last bits and stay within the FP64 oracle's tolerances.
 * It has no reference counterpart. Batches and adjoints require
 * STRO_ARITH_REFERENCE. */
enum { STRO_ARITH_REFERENCE = 0, STRO_ARITH_FUSED = 1 };
int stro_sim_set_arithmetic(stro_sim* sim, int32_t arith);
int stro_sim_get_arithmetic(stro_sim* sim, int32_t* arith);
/* Outflow walls (Cell code 4). STRO_OUTFLOW_DORMANT (default) is the
 * reference's dormant anti-bounce-back: a link to an outflow cell reflects the
 * shifted DDF with its sign flipped (Kernels.metal:28-29, 299-300, 328-329).
 * STRO_OUTFLOW_PRESSURE completes it as a pressure wall at rho_w = 1: the
 * reflected shifted DDF of link i also gains w_i (9 (c_i . u)^2 - 3 u^2), with
 * u = p / rho of the wall cell's gathered DDFs. No reference counterpart; the
 * adjoint requires the dormant wall. */
enum { STRO_OUTFLOW_DORMANT = 0, STRO_OUTFLOW_PRESSURE = 1 };
/* Collision operator. STRO_COLLISION_REFERENCE (default): the reference's
 * SRT / TRT with its sponge, Guo force, Smagorinsky LES and Noble-Torczynski
 * cells. STRO_COLLISION_KBC: the KBC entropic collision (shear part of the
 * non-equilibrium at omega, the rest with the entropic stabiliser), with the
 * sponge and the Guo force; it refuses LES (c_smago > 0) and partially solid
 * cells. No reference counterpart (its roadmap names a cumulant or KBC
 * operator); one-cell kernels only; batches and the adjoint refuse it. */
enum { STRO_COLLISION_REFERENCE = 0, STRO_COLLISION_KBC = 1 };
int stro_sim_set_collision(stro_sim* sim, int32_t collision);
int stro_sim_get_collision(stro_sim* sim, int32_t* collision);
int stro_sim_set_outflow_mode(stro_sim* sim, int32_t mode);
int stro_sim_get_outflow_mode(stro_sim* sim, int32_t* mode);
/* Launch shape of variant 1: bx threads (a multiple of 32 dividing nx/2, at
 * most 256) covering 2*bx cells of one row; by must be 1. */
int stro_sim_set_pair_block(stro_sim* sim, int32_t bx, int32_t by);
int stro_sim_get_pair_block(stro_sim* sim, int32_t* bx, int32_t* by);
/* Kernel path of the latest step launch: "cell" (one cell per thread),
 * "split" (bulk / boundary block lists), "pair", "wide4", "wide8", "rows",
 * "capped" or "probe";
 * "" before the first step. A lattice a variant does not apply to reports the
 * path that ran instead. */
int stro_sim_last_path(stro_sim* sim, char* buf, size_t len);
/* Block counts of the lists the "split" path last ran: bulk (wall-free
 * kernels), x-face and boundary (wall-aware kernels) blocks; all 0 before the
 * split first ran. No reference counterpart. */
int stro_sim_split_blocks(const stro_sim* sim, int64_t* bulk, int64_t* face, int64_t* edge);
/* Launch shape of variant 2: `threads` computing threads per block (a
 * multiple of 32, at most 256; one more warp issues the copies) and `rows`
 * lattice rows per tile (1 to 8). */
int stro_sim_set_rows_tile(stro_sim* sim, int32_t threads, int32_t rows);
int stro_sim_get_rows_tile(stro_sim* sim, int32_t* threads, int32_t* rows);
/* Polls per bounded wait of variant 2 (default 2^22; a bulk copy completes in
 * microseconds). A wait that runs out makes every thread of the block return
 * once the block's copies in flight have landed; the run then fails with
 * STRO_ERR_TIMEOUT and the lattice state is undefined. 0 gives up at the first
 * wait (exercises that path). No reference counterpart. */
int stro_sim_set_spin_limit(stro_sim* sim, int64_t polls);
/* Walled lattices run their bulk blocks (cells with no wall neighbour and no
 * solid fraction) with the wall-free kernels, the blocks whose only walls are
 * velocity-inflow columns at x = 0 and x = nx - 1 with x-face kernels (the
 * wall links follow from x; no geometry is read), and only the other
 * boundary blocks with the wall-aware ones (1, the default); 2 does the same
 * with the boundary blocks' odd pass in column-major cell order (a warp
 * covers whole columns of its block); 3 is 1 without the x-face blocks (they
 * run the wall-aware kernels); 4 is 1 with the bulk and x-face blocks in one
 * launch from one list in block order (a DRAM line shared by an x-face block
 * and the bulk block beside it is fetched once); 5 is 4 with the bulk blocks
 * of an FP16-storage lattice taken two x-adjacent cells per thread in 4-byte
 * words (feature levels without KBC, nx and the block width even; otherwise
 * as 4); 0 runs the wall-aware kernels on every block. Results are identical
 * in every mode. */
int stro_sim_set_block_split(stro_sim* sim, int32_t enabled);
/* stro_sim_run and stro_sim_run_sampled replay CUDA graphs of plain steps once
 * the ramp is over (default on): the launches of a run of steps are captured
 * once per configuration and replayed. 0 launches every step from the host.
 * Results are identical either way. */
int stro_sim_set_graphs(stro_sim* sim, int32_t enabled);
/* Autotuner: times `steps` steps per candidate variant and launch shape on the current
 * state (saved and restored, stepsDone unchanged) and keeps the fastest. */
int stro_sim_autotune(stro_sim* sim, int64_t steps, int32_t* bx, int32_t* by, double* glups);

/* ---- batch: many lattices advanced together ------------------------------------
 * The reference advances credibility-ladder rungs and Mach anchors one after
 * another on one queue (Ladder.swift:74-121). A batch groups simulations of
 * one precision on one context and advances them in one launch. */
typedef struct stro_batch stro_batch;
enum {
    STRO_BATCH_PERSISTENT = 0, /* one cooperative persistent kernel, bounded grid barrier, in a CUDA graph */
    STRO_BATCH_ROUNDS = 1,     /* a CUDA graph of one launch per round */
    STRO_BATCH_SEQUENTIAL = 2, /* one instance after another, one launch per step */
    STRO_BATCH_STREAMS = 3     /* every instance on its own stream with its own kernels and
                                  CUDA graphs, all enqueued before any is waited for */
};
int stro_batch_create(stro_ctx* ctx, int32_t count, stro_sim* const* sims, stro_batch** out);
int stro_batch_destroy(stro_batch* batch);
int stro_batch_set_mode(stro_batch* batch, int32_t mode);
int stro_batch_set_tile(stro_batch* batch, int32_t bx, int32_t by);
/* Polls before a grid-barrier wait gives up with STRO_ERR_TIMEOUT. */
int stro_batch_set_spin_limit(stro_batch* batch, int64_t polls);
/* STRO_BATCH_ROUNDS on simulations with walls or solid fractions: when on (the
 * default) each round runs the tiles whose cells are all plain fluid without
 * wall neighbours on the wall-free kernels and the rest on the wall-aware
 * ones (results bitwise the same). stro_batch_split_tiles reports the last
 * run's bulk and boundary tile counts (0, 0 when it ran unsplit). */
int stro_batch_set_split(stro_batch* batch, int32_t on);
int stro_batch_split_tiles(const stro_batch* batch, int64_t* bulk, int64_t* edge);
/* Advance sims[i] by steps[i] steps (DDFs bitwise identical to stro_sim_run).
 * If log_every != NULL and log_every[i] > 0 (even; sims[i] at an even step
 * count), sum |u|^2 is sampled before the first step and after every
 * log_every[i] steps into traces[i * trace_stride + k]; trace_counts[i] gets
 * the number of samples. */
int stro_batch_run(stro_batch* batch, const int64_t* steps, const int32_t* log_every,
                   double* traces, int32_t trace_stride, int32_t* trace_counts);
/* stro_sim_run_sampled for every simulation of the batch in one submission:
 * instance i takes transient[i] steps, then probes the force over the box
 * boxes[4 i .. 4 i + 3] = {x0, x1, y0, y1} every max(2, stride[i] - 2) + 2
 * steps (rounded as stro_sim_run_sampled does) until sample_steps[i] steps are
 * taken; its samples go to forces[i][3 k + d], at most capacity[i] of them, and
 * their number to samples[i]. DDFs and step counts are bitwise those of
 * stro_sim_run_sampled; the box sums are folded per tile, so forces agree with
 * it to rounding (FP64). In STRO_BATCH_SEQUENTIAL mode the simulations run one
 * after another through stro_sim_run_sampled (the reference's order); in
 * STRO_BATCH_STREAMS mode each runs stro_sim_run_sampled's schedule on its own
 * stream, all at once, and forces equal stro_sim_run_sampled's bit for bit. */
int stro_batch_run_sampled(stro_batch* batch, const int64_t* transient, const int64_t* sample_steps,
                           const int64_t* stride, const int32_t* boxes, double* const* forces,
                           const int64_t* capacity, int64_t* samples);
int stro_batch_gpu_seconds(stro_batch* batch, double* seconds);
/* "persistent-graph", "rounds-graph", "rounds-stream", "sequential" or "streams": the path
 * the last run took. */
int stro_batch_last_path(stro_batch* batch, char* buf, size_t len);
/* Times each mode and tile shape for `rounds` rounds (states restored) and keeps the fastest. */
int stro_batch_autotune(stro_batch* batch, int64_t rounds, int32_t* mode, int32_t* bx,
                        int32_t* by, double* seconds);

/* No counterpart in the reference. Kinetic-energy and dissipation sums (as
 * stro_sim_kinetic_energy / stro_sim_dissipation) of a DDF state the CALLER
 * holds in device memory, for callers that must not allocate: a framework
 * whose own allocator owns the device memory, a real-time loop that cannot
 * afford the implicit synchronisation of cudaMalloc, or code running while a
 * stream is captured. This call allocates nothing. Its scratch is a 32 KB
 * array in the library's device module, present on every GPU that loads the
 * library until exit.
 *   f            device pointer: 19 planes, plane i at f + i*plane_stride elements
 *                (FP32 or FP16 per `precision`)
 *   cell_types   optional device array of N cell bytes; only the low 3 bits are
 *                read, as the Cell code (0 = fluid; cells of other codes are
 *                skipped), so flag bits a caller keeps above them are ignored;
 *                NULL = all fluid
 *   omega        relaxation rate, finite and in (0, 2); others are rejected
 *   force        host pointer to the uniform force (half-force shift of u); NULL = 0
 *   out          device pointer to 2 doubles: sum |u|^2, sum 2 nu S:S (nu from omega)
 *   stream       cudaStream_t (NULL = default stream); the call only enqueues work
 * Lattices up to N < 2^31 cells are accepted; larger ones are rejected with
 * STRO_ERR_INVALID. The first call on a device looks up the scratch address
 * on that device (with it current); make that first call before any stream
 * capture. All calls share the scratch array, so calls whose work overlaps on
 * the GPU (two streams at once) race: order them on one stream. */
int stro_observables_noalloc(const void* f, int32_t precision, int32_t nx, int32_t ny, int32_t nz,
                             uint64_t plane_stride, const uint8_t* cell_types, float omega,
                             const float force[3], double* out, void* stream);

/* ---- discrete adjoint -------------------------------------------------------------
 * No reference counterpart (the reference has no adjoint). Objective over the
 * window [t0, t0 + steps) from the simulation's current state:
 *   J = mean over the odd steps t of dir . F_box(t),
 * F_box = the momentum-exchange force of the odd pass over the cells the
 * reference's probeForce would sum (box x0..x1, y0..y1 inclusive, all z;
 * Sim.swift:359-372): with dir = (1,0,0) the time-averaged drag.
 * stro_adj_forward runs the window (advancing the simulation) and keeps
 * `checkpoints` states on the device; stro_adj_backward recomputes between
 * checkpoints and returns dJ/d eps (N floats: Noble-Torczynski cells, 0 where
 * eps = 0) and dJ/d F_field (3 planes of N floats, the per-cell Guo force). */
typedef struct stro_adjoint stro_adjoint;
int stro_adj_create(stro_sim* sim, const double dir[3], const int32_t box[4], int64_t steps,
                    int32_t checkpoints, stro_adjoint** out);
int stro_adj_destroy(stro_adjoint* adj);
int stro_adj_forward(stro_adjoint* adj, double* J);
int stro_adj_backward(stro_adjoint* adj, float* grad_eps, float* grad_force);
/* Switches the objective to the time-averaged dissipation:
 *   J = mean over m = 1 .. steps / every of D(t0 + m every),
 * D = the dissipation sum of stro_sim_dissipation (2 nu S:S over the fluid
 * cells; the viscous dissipation the reference's Taylor-Green case reads,
 * Cases.swift:1254-1270) of the state after m * every steps. `every` is even
 * and at most the window; the window must start at an even step count
 * (STRO_ERR_STATE otherwise). dir and box are then unused; the gradients keep
 * their meaning (dJ/d F_field includes D's own dependence on the force through
 * u = (p + F/2) / rho). */
int stro_adj_set_dissipation(stro_adjoint* adj, int64_t every);
/* Device seconds of the last forward, of the recomputation and of the adjoint
 * steps, and the number of adjoint steps run. */
int stro_adj_stats(stro_adjoint* adj, double* forward_s, double* recompute_s, double* adjoint_s,
                   int64_t* adjoint_steps);

/* ---- host utilities ---------------------------------------------------------- */
/* SHA-256 (FIPS 180-4) of a host buffer as 64 hex chars + NUL: the digest
 * stro_sim_digest computes over the downloaded state, for caller-held copies. */
int stro_sha256_hex(const void* data, size_t len, char hex[65]);
/* Page-locked host memory for fast state transfers (cudaMallocHost). */
int stro_host_alloc(size_t bytes, void** out);
int stro_host_free(void* ptr);

/* ---- host geometry helpers (CaseSetups.swift) -------------------------------- */
/* diskSolidFractions (CaseSetups.swift:6-25): 16x16 subcell sampling, out = nx*ny floats. */
int stro_disk_solid_fractions(int32_t nx, int32_t ny, double cx, double cy, double r, float* out);
/* sphereSolidFractions (CaseSetups.swift:68-90) with sub^3 subcells per cell
 * (the reference uses sub = 8), out = nx*ny*nz floats. */
int stro_sphere_solid_fractions(int32_t nx, int32_t ny, int32_t nz, double cx, double cy,
                                double cz, double r, int32_t sub, float* out);

/* ---- triangle meshes (StlVoxels.swift) ---------------------------------------
 * StlMesh(binarySTL:) (StlVoxels.swift:11-43): the triangle count of a binary
 * STL, then the triangles (count x 9 floats: three vertices) and the bounds
 * (min xyz, max xyz). Errors as the reference: "STL too short", "ASCII STL not
 * supported (binary only)", "STL truncated (or ASCII; binary only)". */
int stro_stl_triangle_count(const uint8_t* data, size_t len, uint32_t* count);
int stro_stl_parse(const uint8_t* data, size_t len, float* tris, float bounds[6]);
/* sphereSTLData (StlVoxels.swift:120-143): a lat-long sphere as binary STL.
 * With out = NULL only *len (the byte count) is returned. */
int stro_sphere_stl(float radius, int32_t segments, int32_t rings, uint8_t* out, size_t cap,
                    size_t* len);
/* meshSolidFractions (StlVoxels.swift:52-117) on the GPU: Noble-Torczynski
 * fractions of a closed mesh by parity ray casting along +x with 2x2 sub-rays
 * per cell; lattice coordinates = vertex * scale + offset (cell centres at
 * integers). eps: host array of nx*ny*nz floats. seconds (optional): device
 * time of the ray kernel. Fails if one sub-ray crosses the mesh more than 128
 * times. */
int stro_mesh_solid_fractions(stro_ctx* ctx, const float* tris, uint32_t ntri, int32_t nx,
                              int32_t ny, int32_t nz, float scale, const float offset[3],
                              float* eps, double* seconds);

/* ---- uncertainty budget (Uncertainty.swift) ----------------------------------
 * U(phi) = k sqrt(u_num^2 + u_stat^2 + u_Ma^2), k = 2, published only inside
 * or near the edge of the validated domain. Host-only double arithmetic in
 * the reference's operation order. */
typedef struct {
    double mean;          /* mean of the batch means (series mean when too short) */
    double half_width95;  /* u_stat = 1.96 sd / sqrt(batches); NaN when too short */
    double lag1;          /* lag-1 autocorrelation of the batch means */
    int32_t batches;      /* 0 when the series is shorter than 4 * min_batches */
    int32_t trustworthy;  /* batches >= 6 and |lag1| <= 0.3 */
} stro_stat_uq;
/* StatUncertainty(series:maxBatches:minBatches:) (Uncertainty.swift:47-101):
 * non-overlapping batch means, the largest batch count (searching down from
 * max_batches in steps of 2) whose means are uncorrelated (|lag1| <= 0.3). */
int stro_uq_stat(const double* values, int64_t n, int32_t max_batches, int32_t min_batches,
                 stro_stat_uq* out);
typedef struct {
    int32_t cells_per_feature;
    double value; /* time-averaged QoI of the rung */
    double stat;  /* its u_stat (NaN if unknown) */
} stro_ladder_rung;
typedef struct {
    double u_num;          /* max(|finest - next|, finest u_stat); NaN for one rung */
    double observed_order; /* diagnostic only; NaN unless 3 rungs converge monotonically */
    int32_t has_order;
    int32_t note;          /* 0 single resolution, 1 finest two agree within noise, 2 otherwise */
} stro_num_uq;
/* NumUncertainty(rungs:) (Uncertainty.swift:123-163). */
int stro_uq_num(const stro_ladder_rung* rungs, int32_t count, stro_num_uq* out);
/* MachUncertainty (Uncertainty.swift:168-179): u_Ma = 4/3 |baseline - half-Mach|. */
int stro_uq_mach(double baseline, double half_mach, double* u_ma);
enum { STRO_DOMAIN_INSIDE = 0, STRO_DOMAIN_NEAR_EDGE = 1, STRO_DOMAIN_OUTSIDE = 2 };
enum {
    STRO_OUTSIDE_RE = 1, STRO_OUTSIDE_MACH = 2, STRO_OUTSIDE_RESOLUTION = 4,
    STRO_OUTSIDE_GEOMETRY = 8 /* no validated case of that geometry class */
};
typedef struct {
    int32_t verdict;  /* STRO_DOMAIN_* */
    int32_t anchor;   /* nearest anchor of the geometry class, -1 if none */
    double distance;  /* fractional extrapolation distance to it */
    double factor;    /* bar inflation near the edge (1 inside, NaN outside) */
    int32_t reasons;  /* STRO_OUTSIDE_* bits when outside */
} stro_domain_verdict;
/* ValidationDomain.classify (Uncertainty.swift:221-259) over the reference's
 * anchors (Uncertainty.swift:200-213). */
int stro_uq_classify(double re, double mach, int32_t cells_per_feature, const char* geometry,
                     stro_domain_verdict* out);
/* Anchor `index` (0..3): name, ranges {Re lo, Re hi, Ma lo, Ma hi}, cells per
 * feature {lo, hi} and geometry class (UTF-8). */
int stro_uq_anchor(int32_t index, char* name, size_t name_len, double ranges[4],
                   int32_t cells[2], char* geometry, size_t geometry_len);
/* UncertaintyBudget.combined (Uncertainty.swift:272-280): 2 * RSS of the
 * non-NaN components, times the edge factor near the edge, NaN outside. */
int stro_uq_combined(double u_num, double u_stat, double u_ma, const stro_domain_verdict* verdict,
                     double* combined);

#ifdef __cplusplus
}
#endif

#endif /* STROUHAL_C_H */
