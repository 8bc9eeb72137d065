// Internal state of the C-ABI handles, shared by runtime.cu and batch.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "lbm_launch.h"
#include "strouhal_c.h"

struct stro_ctx {
    // Simulations and batches hold a reference; stro_ctx_destroy only marks the
    // context closed and the last holder frees it, so handles may be released
    // in any order.
    int refs = 1;
    bool closed = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    char name[256] = {0};
};

struct stro_sim {
    stro_ctx* ctx = nullptr;
    int precision = STRO_FP32;
    int32_t nx = 0, ny = 0, nz = 0;
    uint64_t N = 0, plane = 0;
    size_t esize = 4;
    // Simulation properties (Sim.swift:164-172)
    float omega = 1.0f, omega_minus = 1.0f;
    float lid[3] = {0, 0, 0};
    float uin = 0.0f;
    int32_t ramp_steps = 0;
    float force[3] = {0, 0, 0};
    float c_smago = 0.0f;
    int inflow_uniform = 0;
    bool sponge_on = false;
    float sponge_x0 = 1e9f, sponge_width = 0.0f, sponge_tau = 1.0f;
    bool wants_forces = false;
    // host geometry
    std::vector<uint8_t> flags;
    std::vector<uint32_t> smask, lmask;
    std::vector<float> eps;
    std::vector<uint8_t> cell_host;   // packed cell bytes, as on the device
    std::vector<uint32_t> geo_host;   // packed geometry words, as on the device
    bool any_wall = false, has_eps = false, has_ffield = false;
    bool ffield_nonzero = false;  // a zero field leaves the step's arithmetic unchanged
    bool force_geometry = false;  // device geometry kept even for an all-fluid lattice
    // device buffers
    void* d_f = nullptr;
    uint8_t* d_cell = nullptr;
    uint32_t* d_geo = nullptr;
    uint32_t* d_lmask = nullptr;
    float* d_eps = nullptr;
    void* d_render = nullptr;     // RGBA binary16 image of the latest rendered slice
    size_t render_bytes = 0;
    float* d_ffield = nullptr;
    float4* d_moments = nullptr;
    double* d_partials = nullptr;
    size_t partials_len = 0;
    double* d_out = nullptr;
    // bookkeeping
    int64_t steps_done = 0;
    double gpu_seconds = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    dim3 block{256, 1, 1};        // launch shape of ordinary steps (autotunable)
    dim3 probe_block{256, 1, 1};  // fixed shape of force-probe steps: fixes the FP64 sum order
    int variant = 0;              // 0: one cell per thread; 1: FP16 x-pairs (lbm_pair.cu);
                                  // 2: rows staged through shared memory (lbm_rows.cu)
                                  // 3: register-capped one cell per thread
    dim3 pair_block{32, 1, 1};    // launch shape of the pair variant (one row per block)
    const char* last_path = "";   // kernel path of the latest step launch (test hook)
    int rows_threads = 256;       // threads per block of the row-staged variant
    int rows_per_tile = 1;        // lattice rows per tile of the row-staged variant
    int arith = 0;                // STRO_ARITH_REFERENCE or STRO_ARITH_FUSED
    int outflow = 0;              // STRO_OUTFLOW_DORMANT or STRO_OUTFLOW_PRESSURE
    int collision = 0;            // STRO_COLLISION_REFERENCE or STRO_COLLISION_KBC
    int* d_error = nullptr;       // device error word of the row-streaming variant
    int64_t rows_polls = 1ll << 22;  // polls per bounded wait of the row-staged variant
    // bulk / boundary block lists of a walled lattice for the current block shape
    bool split = true;
    bool edge_colmajor = false;    // boundary blocks of the odd pass in column-major cell order
    bool face_lists = true;        // x-face blocks on their own kernels (else boundary blocks)
    bool merged_faces = false;     // bulk and x-face blocks in one launch (split mode 4)
    bool pair_bulk = false;        // and FP16 bulk blocks two cells per thread (split mode 5)
    uint32_t* d_blocks = nullptr;  // bulk blocks first, then x-face, then edge blocks
    uint32_t nbulk = 0, nface = 0, nedge = 0;
    bool lists_face = false;       // face_lists when the lists were built
    bool lists_merged = false;     // bulk and x-face blocks in one list (split modes 4 and 5)
    dim3 lists_block{0, 0, 0};
    uint64_t lists_version = ~0ull;
    uint64_t geo_version = 0;      // bumped whenever the device geometry changes
    // CUDA graphs of runs of plain steps, keyed by everything their launches read
    bool graphs = true;
    // Stream of the step launches when not null: a batch in STRO_BATCH_STREAMS
    // mode sets it while it enqueues this lattice's run, then clears it.
    cudaStream_t stream = nullptr;
    std::vector<std::pair<std::vector<uint8_t>, cudaGraphExec_t>> graph_cache;
};

namespace stro {
namespace rt {

// Steps per replayed graph in stro_sim_run (runs of at least twice as many).
constexpr int64_t kRunGraphSteps = 32;

// Stream the step launches of `s` go to.
inline cudaStream_t sim_stream(const stro_sim* s) { return s->stream ? s->stream : s->ctx->stream; }

// A sampled run (stro_sim_run_sampled) in pieces: begin checks the arguments
// and allocates the device sample buffer; each advance enqueues the next piece
// of the schedule (up to 1024 transient steps, or one sample: chunk, probe
// pair, fold) on the simulation's stream without waiting, the last one the
// read-back of the forces; finish waits and does the bookkeeping (or, after
// an error, only frees). A batch interleaves the advances of its instances.
struct SampledRun {
    double* d_samples = nullptr;
    double* forces = nullptr;
    int64_t* steps_at = nullptr;
    int64_t count = 0;           // samples
    int64_t k = 0;               // next sample
    int64_t t = 0;               // step count after what is enqueued
    int64_t transient_left = 0;
    int64_t chunk = 0, g_transient = 0, g_chunk = 0;
    int box[4] = {0, 0, 0, 0};
    bool done = false;           // everything, read-back included, is enqueued
};
int sampled_begin(stro_sim* s, int64_t transient, int64_t sample_steps, int64_t stride,
                  const int32_t box[4], double* forces, int64_t capacity, int64_t* samples,
                  int64_t* steps_at, SampledRun* run);
int sampled_advance(stro_sim* s, SampledRun* run);
int sampled_finish(stro_sim* s, SampledRun* run);

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
bool geo_on(const stro_sim* s);
// Bulk and boundary blocks of the (shape.x, shape.y) block grid of a walled
// lattice (host geometry copies must be current): a bulk block holds only
// fluid cells without wall neighbours or solid fractions. With `face`, the
// boundary blocks that the x-face kernels can take (every wall a
// velocity-inflow cell of the columns x = 0 and x = nx - 1, every link into
// those columns a moving-wall link, no other wall link, no solid fraction) go
// there instead of into `edge`.
void block_lists(const stro_sim* s, dim3 shape, std::vector<uint32_t>& bulk,
                 std::vector<uint32_t>& edge, std::vector<uint32_t>* face = nullptr);
// Feature level of the step kernels: 0 lean, 1 sponge / force / NT, 2 also LES,
// 3 the KBC collision.
int feat_on(const stro_sim* s);
float ramp_factor(const stro_sim* s, int64_t t);
StepArgs step_args(const stro_sim* s, int64_t t);
FieldView field_view(const stro_sim* s);
// Builds the device cell bytes / geometry words even for an all-fluid lattice
// (needed when the lattice joins a batch that runs the wall-aware kernels).
int ensure_geometry(stro_sim* s);
// Launch one lattice step t on the simulation stream (variant and shape of the sim).
cudaError_t launch_sim_step(stro_sim* s, const StepArgs& a, int64_t t, bool probe);
// Launch the plain steps t .. t + count - 1 (no force probe). With graph_steps
// > 0 (even), whole runs of graph_steps steps past the ramp replay one cached
// CUDA graph; everything else is launched step by step. Same kernels, same
// arguments, same results either way.
int launch_plain_steps(stro_sim* s, int64_t t, int64_t count, int64_t graph_steps);
void drop_graphs(stro_sim* s);
// STRO_ERR_TIMEOUT (and the flag reset) if a row-staged step gave up a wait.
int check_rows_error(stro_sim* s);
void ctx_retain(stro_ctx* c);
void ctx_release(stro_ctx* c);
int observables(stro_sim* s, double out[2]);

}  // namespace rt
}  // namespace stro

#define STRO_CUDA(expr)                                              \
    do {                                                             \
        cudaError_t e_ = (expr);                                     \
        if (e_ != cudaSuccess) return ::stro::rt::cuda_fail(e_, #expr); \
    } while (0)
