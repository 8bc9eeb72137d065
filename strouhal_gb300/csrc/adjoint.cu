// Host side of the discrete adjoint (C ABI stro_adj_*): checkpointed forward,
// recomputation between checkpoints, reverse sweep.
//
// The tape is the schedule kept here: the window [t0, t0 + steps), the
// checkpoint states saved every `seg` steps on the device during the forward
// run, and the per-step uniforms (ramp) rebuilt from the step index. The
// backward sweep walks the segments last to first: it restores a segment's
// checkpoint, recomputes the segment forward while keeping every input state
// on the device, then runs the adjoint steps of the segment in reverse.
// Memory: checkpoints + one segment of states (allocated by the first
// backward sweep) + the FP32 adjoint array.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lbm_adjoint.h"
#include "runtime_internal.h"

using namespace stro;
using namespace stro::rt;

struct stro_adjoint {
    stro_sim* sim = nullptr;
    double dir[3] = {1.0, 0.0, 0.0};
    int box[4] = {0, 0, 0, 0};
    int64_t steps = 0, t0 = 0, seg = 0;
    int32_t ncheck = 0;
    bool forward_done = false;
    size_t state_bytes = 0;
    void* d_check = nullptr;   // ncheck states
    void* d_seg = nullptr;     // seg states
    float* d_lam = nullptr;
    double* d_geps = nullptr;  // dJ/d eps, summed in FP64
    float* d_gf = nullptr;
    double* d_forces = nullptr;  // 3 doubles per odd step
    uint32_t* d_lists = nullptr; // bulk blocks, then boundary blocks, of the reverse-step grid
    uint32_t nbulk = 0, nedge = 0;
    int64_t nodd = 0;
    // objective: 0 = mean force over the odd steps; 1 = mean dissipation sum
    // over the states after every, 2 every, ... steps of the window
    int objective = 0;
    int64_t every = 0;
    double* d_diss = nullptr;   // (kinetic energy, dissipation) per sample
    void* d_final = nullptr;    // the window's last state, when it is a sample
    double J = 0.0;
    double fwd_seconds = 0.0, recompute_seconds = 0.0, adjoint_seconds = 0.0;
    int64_t adjoint_launches = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {

void adj_free(stro_adjoint* a) {
    cudaFree(a->d_check);
    cudaFree(a->d_seg);
    cudaFree(a->d_lam);
    cudaFree(a->d_geps);
    cudaFree(a->d_gf);
    cudaFree(a->d_forces);
    cudaFree(a->d_lists);
    cudaFree(a->d_diss);
    cudaFree(a->d_final);
    if (a->e0) cudaEventDestroy(a->e0);
    if (a->e1) cudaEventDestroy(a->e1);
}

char* state_at(void* base, size_t bytes, int64_t k) { return static_cast<char*>(base) + bytes * k; }

int timed(stro_adjoint* a, double* acc, int rc_in) {
    (void)rc_in;
    cudaStream_t st = a->sim->ctx->stream;
    STRO_CUDA(cudaEventRecord(a->e1, st));
    STRO_CUDA(cudaEventSynchronize(a->e1));
    float ms = 0.f;
    STRO_CUDA(cudaEventElapsedTime(&ms, a->e0, a->e1));
    *acc += double(ms) * 1e-3;
    return STRO_OK;
}

// Forward window of the dissipation objective: plain steps (no force probe),
// the observables reduction after every `every` steps into d_diss, and a copy
// of the last state when it is a sample (the reverse sweep injects there
// first). J = mean of the sampled dissipation sums.
int forward_dissipation(stro_adjoint* a) {
    stro_sim* s = a->sim;
    cudaStream_t st = s->ctx->stream;
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "the dissipation objective needs an even step count at the start");
    a->t0 = s->steps_done;
    a->nodd = 0;
    const int64_t K = a->steps / a->every;
    if (!a->d_diss) STRO_CUDA(cudaMalloc(&a->d_diss, size_t(2 * K) * sizeof(double)));
    if (a->steps % a->every == 0 && !a->d_final)
        STRO_CUDA(cudaMalloc(&a->d_final, a->state_bytes));
    const int half = s->precision == STRO_FP16S ? 1 : 0;
    STRO_CUDA(cudaEventRecord(a->e0, st));
    for (int64_t k = 0; k < a->steps; ++k) {
        const int64_t t = a->t0 + k;
        if (k % a->seg == 0)
            STRO_CUDA(cudaMemcpyAsync(state_at(a->d_check, a->state_bytes, k / a->seg), s->d_f,
                                      a->state_bytes, cudaMemcpyDeviceToDevice, st));
        STRO_CUDA(launch_sim_step(s, step_args(s, t), t, false));
        if ((k + 1) % a->every == 0 && (k + 1) / a->every <= K)
            STRO_CUDA(launch_observables(field_view(s), half, s->omega, s->d_partials,
                                         a->d_diss + 2 * ((k + 1) / a->every - 1), st));
    }
    if (a->d_final)
        STRO_CUDA(cudaMemcpyAsync(a->d_final, s->d_f, a->state_bytes, cudaMemcpyDeviceToDevice,
                                  st));
    int rc = timed(a, &a->fwd_seconds, STRO_OK);
    if (rc != STRO_OK) return rc;
    std::vector<double> d(size_t(2 * K));
    STRO_CUDA(cudaMemcpy(d.data(), a->d_diss, d.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double sum = 0.0;
    for (int64_t m = 0; m < K; ++m) sum += d[size_t(2 * m + 1)];
    a->J = sum / double(K);
    s->steps_done += a->steps;
    a->forward_done = true;
    return STRO_OK;
}

// lam += w dD/df at the sampled state `state` (see launch_adjoint_dissipation).
int inject_dissipation(stro_adjoint* a, const void* state, int64_t t) {
    stro_sim* s = a->sim;
    AdjArgs g{};
    g.a = step_args(s, t);
    g.a.f = const_cast<void*>(state);
    g.a.ffield_plane = uint32_t(s->N);
    g.lam = a->d_lam;
    g.grad_f = a->d_gf;
    const float nu = float((1.0 / double(s->omega) - 0.5) / 3.0);
    const float w = float(1.0 / double(a->steps / a->every));
    STRO_CUDA(launch_adjoint_dissipation(g, s->precision == STRO_FP16S ? 1 : 0, nu, w,
                                         s->ctx->stream));
    return STRO_OK;
}

}  // namespace

extern "C" {

int stro_adj_create(stro_sim* s, const double dir[3], const int32_t box[4], int64_t steps,
                    int32_t checkpoints, stro_adjoint** out) {
    if (!s || !dir || !box || !out) return fail(STRO_ERR_INVALID, "null argument");
    *out = nullptr;
    if (steps < 1) return fail(STRO_ERR_INVALID, "the window needs at least one step");
    if (s->arith != STRO_ARITH_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference arithmetic only");
    if (s->outflow != STRO_OUTFLOW_DORMANT)
        return fail(STRO_ERR_INVALID, "the adjoint covers the dormant outflow wall only");
    if (s->collision != STRO_COLLISION_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference collision only");
    if (checkpoints < 1) checkpoints = 1;
    if (checkpoints > steps) checkpoints = int32_t(steps);
    if (box[0] < 0 || box[1] >= s->nx || box[2] < 0 || box[3] >= s->ny || box[0] > box[1] ||
        box[2] > box[3])
        return fail(STRO_ERR_INVALID, "force box outside the lattice");
    cudaSetDevice(s->ctx->device);
    stro_adjoint* a = new (std::nothrow) stro_adjoint;
    if (!a) return fail(STRO_ERR_OOM, "host allocation failed");
    a->sim = s;
    std::memcpy(a->dir, dir, sizeof a->dir);
    std::memcpy(a->box, box, sizeof a->box);
    a->steps = steps;
    a->ncheck = checkpoints;
    a->seg = (steps + checkpoints - 1) / checkpoints;
    a->state_bytes = 19 * s->plane * s->esize;
    const uint64_t N = s->N;
    cudaError_t e = cudaMalloc(&a->d_check, a->state_bytes * size_t(a->ncheck));
    if (e == cudaSuccess) e = cudaMalloc(&a->d_lam, 19 * s->plane * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&a->d_geps, N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&a->d_gf, 3 * N * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&a->d_forces, size_t(steps / 2 + 2) * 3 * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&a->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&a->e1);
    if (e != cudaSuccess) {
        adj_free(a);
        delete a;
        return cuda_fail(e, "adjoint buffers");
    }
    *out = a;
    return STRO_OK;
}

int stro_adj_destroy(stro_adjoint* a) {
    if (!a) return STRO_OK;
    cudaSetDevice(a->sim->ctx->device);
    cudaStreamSynchronize(a->sim->ctx->stream);
    adj_free(a);
    delete a;
    return STRO_OK;
}

int stro_adj_set_dissipation(stro_adjoint* a, int64_t every) {
    if (!a) return fail(STRO_ERR_INVALID, "null adjoint handle");
    if (every < 2 || every % 2 != 0 || every > a->steps)
        return fail(STRO_ERR_INVALID, "the sample interval must be even and within the window");
    a->objective = 1;
    a->every = every;
    a->forward_done = false;
    cudaSetDevice(a->sim->ctx->device);
    cudaFree(a->d_diss);
    cudaFree(a->d_final);
    a->d_diss = nullptr;
    a->d_final = nullptr;
    return STRO_OK;
}

int stro_adj_forward(stro_adjoint* a, double* J) {
    if (!a || !J) return fail(STRO_ERR_INVALID, "null argument");
    stro_sim* s = a->sim;
    if (s->arith != STRO_ARITH_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference arithmetic only");
    if (s->outflow != STRO_OUTFLOW_DORMANT)
        return fail(STRO_ERR_INVALID, "the adjoint covers the dormant outflow wall only");
    if (s->collision != STRO_COLLISION_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference collision only");
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    if (a->objective == 1) {
        const int rc = forward_dissipation(a);
        if (rc == STRO_OK) *J = a->J;
        return rc;
    }
    a->t0 = s->steps_done;
    a->nodd = 0;
    const bool geo = geo_on(s);
    if (geo) {
        const dim3 g = step_grid(step_args(s, 0), s->probe_block);
        const size_t need = size_t(3) * g.x * g.y * g.z;
        if (s->partials_len < need) {
            cudaFree(s->d_partials);
            s->d_partials = nullptr;
            s->partials_len = 0;
            STRO_CUDA(cudaMalloc(&s->d_partials, need * sizeof(double)));
            s->partials_len = need;
        }
    }
    STRO_CUDA(cudaEventRecord(a->e0, st));
    for (int64_t k = 0; k < a->steps; ++k) {
        const int64_t t = a->t0 + k;
        if (k % a->seg == 0)
            STRO_CUDA(cudaMemcpyAsync(state_at(a->d_check, a->state_bytes, k / a->seg), s->d_f,
                                      a->state_bytes, cudaMemcpyDeviceToDevice, st));
        StepArgs sa = step_args(s, t);
        const bool odd = (t & 1) != 0;
        const bool probe = odd && geo;
        if (probe) {
            sa.box_x0 = a->box[0]; sa.box_x1 = a->box[1];
            sa.box_y0 = a->box[2]; sa.box_y1 = a->box[3];
        }
        STRO_CUDA(launch_sim_step(s, sa, t, probe));
        if (odd) {
            if (probe) {
                const dim3 g = step_grid(sa, s->probe_block);
                STRO_CUDA(launch_fold(s->d_partials, int(g.x * g.y * g.z), 3,
                                      a->d_forces + 3 * a->nodd, st));
            } else {
                STRO_CUDA(cudaMemsetAsync(a->d_forces + 3 * a->nodd, 0, 3 * sizeof(double), st));
            }
            ++a->nodd;
        }
    }
    int rc = timed(a, &a->fwd_seconds, STRO_OK);
    if (rc != STRO_OK) return rc;
    std::vector<double> forces(size_t(3 * a->nodd));
    if (a->nodd)
        STRO_CUDA(cudaMemcpy(forces.data(), a->d_forces, forces.size() * sizeof(double),
                             cudaMemcpyDeviceToHost));
    double sum = 0.0;
    for (int64_t j = 0; j < a->nodd; ++j)
        sum += a->dir[0] * forces[3 * j] + a->dir[1] * forces[3 * j + 1] +
               a->dir[2] * forces[3 * j + 2];
    a->J = a->nodd ? sum / double(a->nodd) : 0.0;
    s->steps_done += a->steps;
    a->forward_done = true;
    *J = a->J;
    return STRO_OK;
}

int stro_adj_backward(stro_adjoint* a, float* grad_eps, float* grad_force) {
    if (!a) return fail(STRO_ERR_INVALID, "null adjoint handle");
    if (!a->forward_done) return fail(STRO_ERR_STATE, "stro_adj_forward must run first");
    stro_sim* s = a->sim;
    if (s->arith != STRO_ARITH_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference arithmetic only");
    if (s->outflow != STRO_OUTFLOW_DORMANT)
        return fail(STRO_ERR_INVALID, "the adjoint covers the dormant outflow wall only");
    if (s->collision != STRO_COLLISION_REFERENCE)
        return fail(STRO_ERR_INVALID, "the adjoint differentiates the reference collision only");
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    const uint64_t N = s->N;
    const int half = s->precision == STRO_FP16S ? 1 : 0;
    if (!a->d_seg)  // the segment of recomputed states is only needed by the reverse sweep
        STRO_CUDA(cudaMalloc(&a->d_seg, a->state_bytes * size_t(a->seg)));
    const int geo = geo_on(s) ? 1 : 0;
    STRO_CUDA(cudaMemsetAsync(a->d_lam, 0, 19 * s->plane * sizeof(float), st));
    STRO_CUDA(cudaMemsetAsync(a->d_geps, 0, N * sizeof(double), st));
    STRO_CUDA(cudaMemsetAsync(a->d_gf, 0, 3 * N * sizeof(float), st));
    const bool diss = a->objective == 1;
    const float w = (!diss && a->nodd) ? float(1.0 / double(a->nodd)) : 0.0f;
    if (diss && a->d_final) {  // the last state is a sample: its gradient starts the sweep
        const int rc = inject_dissipation(a, a->d_final, a->t0 + a->steps);
        if (rc != STRO_OK) return rc;
    }
    const dim3 ablock(32, 4, 1);
    // walled lattice: bulk blocks take the wall-free reverse step, as the forward split does
    const bool split = geo && s->split && s->geo_host.size() == N;
    if (split) {  // from the geometry as it is now
        // as the step's block lists: no launch still reads the old buffer, and
        // the upload is ordered on this stream ahead of the reverse steps
        STRO_CUDA(cudaStreamSynchronize(st));
        cudaFree(a->d_lists);
        a->d_lists = nullptr;
        std::vector<uint32_t> bulk, edge;
        block_lists(s, ablock, bulk, edge);
        a->nbulk = uint32_t(bulk.size());
        a->nedge = uint32_t(edge.size());
        bulk.insert(bulk.end(), edge.begin(), edge.end());
        STRO_CUDA(cudaMalloc(&a->d_lists, std::max<size_t>(bulk.size(), 1) * sizeof(uint32_t)));
        STRO_CUDA(cudaMemcpyAsync(a->d_lists, bulk.data(), bulk.size() * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, st));
        STRO_CUDA(cudaStreamSynchronize(st));
    }
    // the forward kernels step the buffer a StepArgs points to: the recomputation
    // below steps the segment buffers, never the simulation's own state
    for (int32_t c = a->ncheck - 1; c >= 0; --c) {
        const int64_t k0 = int64_t(c) * a->seg;
        const int64_t len = std::min<int64_t>(a->seg, a->steps - k0);
        if (len <= 0) continue;
        // recompute the segment, keeping the input state of every step
        STRO_CUDA(cudaEventRecord(a->e0, st));
        STRO_CUDA(cudaMemcpyAsync(state_at(a->d_seg, a->state_bytes, 0),
                                  state_at(a->d_check, a->state_bytes, c), a->state_bytes,
                                  cudaMemcpyDeviceToDevice, st));
        for (int64_t k = 1; k < len; ++k) {
            void* cur = state_at(a->d_seg, a->state_bytes, k);
            void* prev = state_at(a->d_seg, a->state_bytes, k - 1);
            StepArgs sa = step_args(s, a->t0 + k0 + k - 1);
            if (geo) {
                // walled lattices run one-cell or block-list kernels, which can
                // write the pass out of place: no copy of the previous state
                sa.f = prev;
                sa.f_out = cur;
            } else {
                STRO_CUDA(cudaMemcpyAsync(cur, prev, a->state_bytes, cudaMemcpyDeviceToDevice,
                                          st));
                sa.f = cur;
            }
            STRO_CUDA(launch_sim_step(s, sa, a->t0 + k0 + k - 1, false));
        }
        int rc = timed(a, &a->recompute_seconds, STRO_OK);
        if (rc != STRO_OK) return rc;
        // adjoint steps of the segment, last to first
        STRO_CUDA(cudaEventRecord(a->e0, st));
        for (int64_t k = len - 1; k >= 0; --k) {
            const int64_t t = a->t0 + k0 + k;
            AdjArgs g{};
            g.a = step_args(s, t);
            g.a.f = state_at(a->d_seg, a->state_bytes, k);
            g.a.ffield_plane = uint32_t(N);
            g.lam = a->d_lam;
            g.grad_eps = a->d_geps;
            g.grad_f = a->d_gf;
            g.obj_w = (t & 1) ? w : 0.0f;
            for (int q = 0; q < 3; ++q) g.dir[q] = float(a->dir[q]);
            std::memcpy(g.box, a->box, sizeof g.box);
            g.force_terms = 1;
            if (split)
                STRO_CUDA(launch_adjoint_split(g, half, int(t & 1), ablock, a->d_lists, a->nbulk,
                                               a->d_lists + a->nbulk, a->nedge, st));
            else
                STRO_CUDA(launch_adjoint_step(g, half, int(t & 1), geo, ablock, st));
            ++a->adjoint_launches;
            // lam is now the adjoint of the state after t - t0 steps of the window
            if (diss && t > a->t0 && (t - a->t0) % a->every == 0) {
                const int irc = inject_dissipation(a, g.a.f, t);
                if (irc != STRO_OK) return irc;
            }
        }
        rc = timed(a, &a->adjoint_seconds, STRO_OK);
        if (rc != STRO_OK) return rc;
    }
    if (grad_eps) {
        std::vector<double> ge(N);
        STRO_CUDA(cudaMemcpyAsync(ge.data(), a->d_geps, N * sizeof(double), cudaMemcpyDeviceToHost,
                                  st));
        STRO_CUDA(cudaStreamSynchronize(st));
        for (uint64_t k = 0; k < N; ++k) grad_eps[k] = float(ge[k]);
    }
    if (grad_force) {
        STRO_CUDA(cudaMemcpyAsync(grad_force, a->d_gf, 3 * N * sizeof(float),
                                  cudaMemcpyDeviceToHost, st));
        STRO_CUDA(cudaStreamSynchronize(st));
    }
    return STRO_OK;
}

int stro_adj_stats(stro_adjoint* a, double* forward_s, double* recompute_s, double* adjoint_s,
                   int64_t* adjoint_steps) {
    if (!a) return fail(STRO_ERR_INVALID, "null adjoint handle");
    if (forward_s) *forward_s = a->fwd_seconds;
    if (recompute_s) *recompute_s = a->recompute_seconds;
    if (adjoint_s) *adjoint_s = a->adjoint_seconds;
    if (adjoint_steps) *adjoint_steps = a->adjoint_launches;
    return STRO_OK;
}

}  // extern "C"
