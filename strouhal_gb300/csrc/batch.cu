// Host side of batched stepping (C ABI stro_batch_*) and the launch-shape
// autotuners.
//
// A batch groups existing simulations of one precision on one context. A run
// advances instance i by steps[i] lattice steps, exactly as calling
// stro_sim_run on each in turn would (same kernels, bitwise identical DDFs),
// but in one launch:
//   STRO_BATCH_PERSISTENT  one cooperative persistent kernel with a bounded
//                          grid barrier between rounds, captured in a CUDA
//                          graph together with the reset of its control word;
//   STRO_BATCH_ROUNDS      a CUDA graph of one launch per round;
//   STRO_BATCH_SEQUENTIAL  the reference's order: one instance after another,
//                          one launch per step (the baseline the batch is
//                          measured against).
// The instantiated graph is cached and replayed while the schedule (step
// counts, logging, tile shape) is unchanged; the per-instance descriptors are
// re-uploaded before every replay.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "lbm_batch.h"
#include "runtime_internal.h"

using namespace stro;
using namespace stro::rt;

struct stro_batch {
    stro_ctx* ctx = nullptr;
    std::vector<stro_sim*> sims;
    int mode = STRO_BATCH_PERSISTENT;
    dim3 block{32, 8, 1};
    int half = 0;
    double gpu_seconds = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    BatchInstance* d_inst = nullptr;
    size_t inst_cap = 0;
    double* d_kepart = nullptr;
    size_t kepart_cap = 0;
    BatchCtl* d_ctl = nullptr;
    float* d_ramp = nullptr;
    size_t ramp_cap = 0;
    double* d_traces = nullptr;
    size_t traces_cap = 0;
    long long spin_limit = 20000000;  // ~2 s of 64 ns polls per barrier wait
    cudaGraphExec_t exec = nullptr;
    std::vector<int64_t> exec_key;
    std::string last_path;
    int64_t last_rounds = 0;
};

namespace {

template <typename T>
int grow(T** p, size_t* cap, size_t n) {
    if (*cap >= n) return STRO_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    STRO_CUDA(cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T)));
    *cap = n;
    return STRO_OK;
}

void drop_graph(stro_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->exec_key.clear();
}

bool batch_geo(const stro_batch* b) {
    for (auto* s : b->sims)
        if (geo_on(s)) return true;
    return false;
}
int batch_feat(const stro_batch* b) {
    int level = 0;
    for (auto* s : b->sims) level = std::max(level, feat_on(s));
    return level;
}

// The reference's order: instance after instance, step after step.
int run_sequential(stro_batch* b, const int64_t* steps, const int32_t* log_every,
                   std::vector<std::vector<double>>& traces) {
    for (size_t i = 0; i < b->sims.size(); ++i) {
        stro_sim* s = b->sims[i];
        const int64_t le = log_every ? log_every[i] : 0;
        int64_t left = steps[i];
        if (le > 0) {
            double o[2];
            int rc = observables(s, o);
            if (rc != STRO_OK) return rc;
            traces[i].push_back(o[0]);
            while (left > 0) {
                const int64_t k = std::min<int64_t>(le, left);
                rc = stro_sim_run(s, k);
                if (rc != STRO_OK) return rc;
                left -= k;
                if (k == le) {
                    rc = observables(s, o);
                    if (rc != STRO_OK) return rc;
                    traces[i].push_back(o[0]);
                }
            }
        } else if (left > 0) {
            const int rc = stro_sim_run(s, left);
            if (rc != STRO_OK) return rc;
        }
    }
    return STRO_OK;
}

int run_fused(stro_batch* b, const int64_t* steps, const int32_t* log_every,
              std::vector<std::vector<double>>& traces) {
    const size_t n = b->sims.size();
    cudaStream_t st = b->ctx->stream;
    const int geo = batch_geo(b) ? 1 : 0;
    const int feat = batch_feat(b);
    if (geo)
        for (auto* s : b->sims) {
            const int rc = ensure_geometry(s);
            if (rc != STRO_OK) return rc;
        }
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), size_t(0));
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t p, size_t q) { return steps[p] > steps[q]; });
    std::vector<BatchInstance> inst(n);
    std::vector<float> ramp;
    std::vector<size_t> ramp_off(n, size_t(-1)), trace_off(n, 0);
    size_t tiles = 0, trace_total = 0;
    int64_t max_steps = 0;
    for (size_t k = 0; k < n; ++k) {
        stro_sim* s = b->sims[order[k]];
        BatchInstance& I = inst[k];
        std::memset(&I, 0, sizeof I);
        I.a = step_args(s, s->steps_done);
        I.t0 = s->steps_done;
        I.steps = steps[order[k]];
        I.log_every = log_every ? log_every[order[k]] : 0;
        I.uin_target = s->uin;
        std::memcpy(I.lid_target, s->lid, sizeof I.lid_target);
        if (s->ramp_steps > 0 && s->steps_done < s->ramp_steps) {
            ramp_off[k] = ramp.size();
            for (int64_t r = 0; r < I.steps; ++r) ramp.push_back(ramp_factor(s, I.t0 + r));
        }
        const uint32_t threads = b->block.x * b->block.y;
        I.cells = uint32_t(s->N);
        I.ntiles = (I.cells + threads - 1) / threads;
        I.tile_begin = uint32_t(tiles);
        tiles += I.ntiles;
        if (I.log_every > 0) {
            I.trace_cap = int32_t((I.steps + I.log_every - 1) / I.log_every);
            trace_off[k] = trace_total;
            trace_total += size_t(I.trace_cap);
        }
        max_steps = std::max(max_steps, I.steps);
    }
    if (tiles >= (1ull << 31)) return fail(STRO_ERR_INVALID, "batch too large");
    int rc = grow(&b->d_inst, &b->inst_cap, n);
    if (rc == STRO_OK) rc = grow(&b->d_kepart, &b->kepart_cap, tiles);
    if (rc == STRO_OK) rc = grow(&b->d_ramp, &b->ramp_cap, ramp.size());
    if (rc == STRO_OK) rc = grow(&b->d_traces, &b->traces_cap, trace_total);
    if (rc == STRO_OK && !b->d_ctl) STRO_CUDA(cudaMalloc(&b->d_ctl, sizeof(BatchCtl)));
    if (rc != STRO_OK) return rc;
    for (size_t k = 0; k < n; ++k) {
        inst[k].ramp = ramp_off[k] == size_t(-1) ? nullptr : b->d_ramp + ramp_off[k];
        inst[k].trace = inst[k].log_every > 0 ? b->d_traces + trace_off[k] : nullptr;
    }
    STRO_CUDA(cudaMemcpyAsync(b->d_inst, inst.data(), n * sizeof(BatchInstance),
                              cudaMemcpyHostToDevice, st));
    if (!ramp.empty())
        STRO_CUDA(cudaMemcpyAsync(b->d_ramp, ramp.data(), ramp.size() * sizeof(float),
                                  cudaMemcpyHostToDevice, st));
    BatchArgs args{};
    args.inst = b->d_inst;
    args.count = int32_t(n);
    args.max_steps = max_steps;
    args.kepart = b->d_kepart;
    args.ctl = b->d_ctl;
    args.spin_limit = b->spin_limit;

    // schedule key of the cached graph
    std::vector<int64_t> key = {b->mode, int64_t(b->block.x), int64_t(b->block.y), geo, feat,
                                b->half, int64_t(n), max_steps, int64_t(tiles),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_inst)),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_kepart)),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_ctl))};
    for (size_t k = 0; k < n; ++k) {
        key.push_back(inst[k].steps);
        key.push_back(inst[k].log_every);
        key.push_back(inst[k].ntiles);
        key.push_back(inst[k].t0 & 1);
    }
    unsigned grid = 0;
    if (b->mode == STRO_BATCH_PERSISTENT) {
        const int per_sm = batch_persistent_blocks_per_sm(b->half, geo, feat, b->block);
        if (per_sm <= 0) return fail(STRO_ERR_CUDA, "persistent kernel cannot be resident");
        grid = unsigned(std::min<size_t>(tiles, size_t(per_sm) * b->ctx->sm_count));
        if (grid == 0) grid = 1;
        key.push_back(grid);
    }
    if (key != b->exec_key) {
        drop_graph(b);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
        cudaError_t le = cudaSuccess;
        if (b->mode == STRO_BATCH_PERSISTENT) {
            le = cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchCtl), st);
            if (le == cudaSuccess)
                le = launch_batch_persistent(args, b->half, geo, feat, grid, b->block, st);
        } else {
            for (int64_t r = 0; r < max_steps && le == cudaSuccess; ++r) {
                uint32_t active = 0;
                bool logs = false;
                for (size_t k = 0; k < n; ++k) {
                    if (inst[k].steps <= r) break;
                    active = inst[k].tile_begin + inst[k].ntiles;
                    if (inst[k].log_every > 0 && r % inst[k].log_every == 0 &&
                        ((inst[k].t0 + r) & 1) == 0)
                        logs = true;
                }
                le = launch_batch_round(args, b->half, geo, feat, r, active, b->block, st);
                if (le == cudaSuccess && logs) le = launch_batch_fold(args, r, st);
            }
        }
        e = cudaStreamEndCapture(st, &graph);
        if (le != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cuda_fail(le, "batch launch (capture)");
        }
        if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
        e = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cuda_fail(e, "batch graph instantiate");
        }
        b->exec_key = key;
    }
    b->last_path = b->mode == STRO_BATCH_PERSISTENT ? "persistent-graph" : "rounds-graph";
    b->last_rounds = max_steps;
    STRO_CUDA(cudaGraphLaunch(b->exec, st));
    BatchCtl ctl{};
    STRO_CUDA(cudaMemcpyAsync(&ctl, b->d_ctl, sizeof ctl, cudaMemcpyDeviceToHost, st));
    STRO_CUDA(cudaStreamSynchronize(st));
    if (b->mode == STRO_BATCH_PERSISTENT && ctl.error != 0)
        return fail(STRO_ERR_TIMEOUT, "batch grid barrier wait timed out at round " +
                                          std::to_string(ctl.error_round));
    std::vector<double> host(trace_total);
    if (trace_total)
        STRO_CUDA(cudaMemcpy(host.data(), b->d_traces, trace_total * sizeof(double),
                             cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < n; ++k) {
        const size_t i = order[k];
        stro_sim* s = b->sims[i];
        s->steps_done += inst[k].steps;
        if (inst[k].log_every > 0) {
            traces[i].assign(host.begin() + trace_off[k],
                             host.begin() + trace_off[k] + inst[k].trace_cap);
            if (inst[k].steps % inst[k].log_every == 0) {
                double o[2];
                const int orc = observables(s, o);
                if (orc != STRO_OK) return orc;
                traces[i].push_back(o[0]);
            }
        }
    }
    return STRO_OK;
}

int tune_sim_shape(stro_sim* s, int64_t steps, int variant, dim3 cand, double* seconds) {
    cudaStream_t st = s->ctx->stream;
    const dim3 saved = s->block, saved_pair = s->pair_block;
    const int saved_variant = s->variant, saved_rows = s->rows_threads,
              saved_tile = s->rows_per_tile;
    s->variant = variant;
    if (variant == 1) {
        s->pair_block = cand;
    } else if (variant == 2) {  // (threads, rows per tile)
        s->rows_threads = int(cand.x);
        s->rows_per_tile = int(cand.y);
    } else {
        s->block = cand;  // variants 0 and 3
    }
    const int64_t t0 = s->steps_done;
    const double g0 = s->gpu_seconds;
    // warm-up pair, then the timed steps
    StepArgs a = step_args(s, t0);
    cudaError_t e = launch_sim_step(s, a, t0, false);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev0, st);
    for (int64_t k = 1; k <= steps && e == cudaSuccess; ++k) {
        a = step_args(s, t0 + k);
        e = launch_sim_step(s, a, t0 + k, false);
    }
    if (e == cudaSuccess) e = cudaEventRecord(s->ev1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(s->ev1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    int err = 0;
    if (e == cudaSuccess && variant == 2)
        e = cudaMemcpy(&err, s->d_error, sizeof err, cudaMemcpyDeviceToHost);
    s->block = saved;
    s->pair_block = saved_pair;
    s->variant = saved_variant;
    s->rows_threads = saved_rows;
    s->rows_per_tile = saved_tile;
    s->gpu_seconds = g0;
    if (e != cudaSuccess) return cuda_fail(e, "autotune launch");
    if (err != 0) {
        cudaMemset(s->d_error, 0, sizeof(int));
        return fail(STRO_ERR_TIMEOUT, "a bulk-copy wait of the row-staged step timed out");
    }
    *seconds = double(ms) * 1e-3;
    return STRO_OK;
}

const dim3 kShapes[] = {dim3(32, 8, 1), dim3(64, 4, 1), dim3(128, 2, 1), dim3(256, 1, 1),
                        dim3(16, 16, 1), dim3(32, 4, 1), dim3(64, 2, 1), dim3(128, 1, 1),
                        dim3(16, 8, 1), dim3(64, 1, 1), dim3(96, 1, 1), dim3(192, 1, 1),
                        dim3(32, 1, 1)};
// (threads, rows per tile) of the row-staged variant
const dim3 kRowShapes[] = {dim3(128, 1, 1), dim3(256, 1, 1), dim3(128, 2, 1), dim3(256, 2, 1),
                           dim3(256, 4, 1), dim3(64, 1, 1)};

}  // namespace

extern "C" {

int stro_batch_create(stro_ctx* ctx, int32_t count, stro_sim* const* sims, stro_batch** out) {
    if (!ctx || !sims || !out || count < 1) return fail(STRO_ERR_INVALID, "bad batch arguments");
    *out = nullptr;
    for (int32_t i = 0; i < count; ++i) {
        if (!sims[i]) return fail(STRO_ERR_INVALID, "null simulation in batch");
        if (sims[i]->ctx != ctx) return fail(STRO_ERR_INVALID, "batch spans contexts");
        if (sims[i]->precision != sims[0]->precision)
            return fail(STRO_ERR_INVALID, "batch mixes precisions");
        if (sims[i]->arith != STRO_ARITH_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference arithmetic only");
        for (int32_t j = 0; j < i; ++j)
            if (sims[j] == sims[i]) return fail(STRO_ERR_INVALID, "simulation listed twice");
    }
    cudaSetDevice(ctx->device);
    stro_batch* b = new (std::nothrow) stro_batch;
    if (!b) return fail(STRO_ERR_OOM, "host allocation failed");
    if (ctx->closed) {
        delete b;
        return fail(STRO_ERR_INVALID, "context already destroyed");
    }
    b->ctx = ctx;
    b->sims.assign(sims, sims + count);
    b->half = sims[0]->precision == STRO_FP16S ? 1 : 0;
    cudaError_t e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "batch events");
    }
    ctx_retain(ctx);
    *out = b;
    return STRO_OK;
}

int stro_batch_destroy(stro_batch* b) {
    if (!b) return STRO_OK;
    stro_ctx* c = b->ctx;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    drop_graph(b);
    cudaFree(b->d_inst);
    cudaFree(b->d_kepart);
    cudaFree(b->d_ctl);
    cudaFree(b->d_ramp);
    cudaFree(b->d_traces);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    ctx_release(c);
    return STRO_OK;
}

int stro_batch_set_mode(stro_batch* b, int32_t mode) {
    if (!b) return fail(STRO_ERR_INVALID, "null batch");
    if (mode != STRO_BATCH_PERSISTENT && mode != STRO_BATCH_ROUNDS && mode != STRO_BATCH_SEQUENTIAL)
        return fail(STRO_ERR_INVALID, "unknown batch mode");
    b->mode = mode;
    return STRO_OK;
}

int stro_batch_set_tile(stro_batch* b, int32_t bx, int32_t by) {
    if (!b) return fail(STRO_ERR_INVALID, "null batch");
    if (bx < 1 || by < 1 || bx * by > 256 || (bx * by) % 32 != 0)
        return fail(STRO_ERR_INVALID, "tile must have a multiple of 32 threads, at most 256");
    b->block = dim3(bx, by, 1);
    return STRO_OK;
}

int stro_batch_set_spin_limit(stro_batch* b, int64_t polls) {
    if (!b || polls < 1) return fail(STRO_ERR_INVALID, "bad spin limit");
    b->spin_limit = polls;
    drop_graph(b);
    return STRO_OK;
}

int stro_batch_run(stro_batch* b, const int64_t* steps, const int32_t* log_every, double* traces,
                   int32_t trace_stride, int32_t* trace_counts) {
    if (!b || !steps) return fail(STRO_ERR_INVALID, "null argument");
    const size_t n = b->sims.size();
    for (size_t i = 0; i < n; ++i) {
        if (steps[i] < 0) return fail(STRO_ERR_INVALID, "negative step count");
        if (b->sims[i]->arith != STRO_ARITH_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference arithmetic only");
        if (log_every && log_every[i] != 0) {
            if (log_every[i] < 0 || log_every[i] % 2 != 0)
                return fail(STRO_ERR_INVALID, "log_every must be even");
            if (b->sims[i]->steps_done % 2 != 0)
                return fail(STRO_ERR_STATE, "logging requires an even step count");
            if (!traces || !trace_counts) return fail(STRO_ERR_INVALID, "trace buffers missing");
        }
    }
    cudaSetDevice(b->ctx->device);
    std::vector<std::vector<double>> tr(n);
    cudaStream_t st = b->ctx->stream;
    STRO_CUDA(cudaEventRecord(b->ev0, st));
    int rc;
    if (b->mode == STRO_BATCH_SEQUENTIAL) {
        rc = run_sequential(b, steps, log_every, tr);
        b->last_path = "sequential";
    } else {
        rc = run_fused(b, steps, log_every, tr);
    }
    if (rc != STRO_OK) return rc;
    STRO_CUDA(cudaEventRecord(b->ev1, st));
    STRO_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.0f;
    STRO_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->gpu_seconds += double(ms) * 1e-3;
    if (log_every) {
        for (size_t i = 0; i < n; ++i) {
            if (log_every[i] == 0) {
                if (trace_counts) trace_counts[i] = 0;
                continue;
            }
            const size_t c = std::min<size_t>(tr[i].size(), size_t(std::max(trace_stride, 0)));
            std::copy(tr[i].begin(), tr[i].begin() + c, traces + i * size_t(trace_stride));
            trace_counts[i] = int32_t(tr[i].size());
        }
    }
    return STRO_OK;
}

int stro_batch_gpu_seconds(stro_batch* b, double* seconds) {
    if (!b || !seconds) return fail(STRO_ERR_INVALID, "null argument");
    *seconds = b->gpu_seconds;
    return STRO_OK;
}

int stro_batch_last_path(stro_batch* b, char* buf, size_t len) {
    if (!b || !buf || !len) return fail(STRO_ERR_INVALID, "null argument");
    std::snprintf(buf, len, "%s", b->last_path.c_str());
    return STRO_OK;
}

int stro_sim_set_block(stro_sim* s, int32_t bx, int32_t by) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (bx < 1 || by < 1 || bx * by > 256 || (bx * by) % 32 != 0)
        return fail(STRO_ERR_INVALID, "block must have a multiple of 32 threads, at most 256");
    s->block = dim3(bx, by, 1);
    return STRO_OK;
}

int stro_sim_set_variant(stro_sim* s, int32_t variant) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (variant < 0 || variant > 3) return fail(STRO_ERR_INVALID, "variant must be 0..3");
    s->variant = variant;
    return STRO_OK;
}

int stro_sim_set_block_split(stro_sim* s, int32_t enabled) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    s->split = enabled != 0;
    return STRO_OK;
}

int stro_sim_set_pair_block(stro_sim* s, int32_t bx, int32_t by) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (bx < 32 || bx > 256 || bx % 32 != 0 || by != 1)
        return fail(STRO_ERR_INVALID, "pair block: bx a multiple of 32 up to 256, by = 1");
    s->pair_block = dim3(bx, by, 1);
    return STRO_OK;
}

int stro_sim_get_pair_block(stro_sim* s, int32_t* bx, int32_t* by) {
    if (!s || !bx || !by) return fail(STRO_ERR_INVALID, "null argument");
    *bx = int32_t(s->pair_block.x);
    *by = int32_t(s->pair_block.y);
    return STRO_OK;
}

int stro_sim_last_path(stro_sim* s, char* buf, size_t len) {
    if (!s || !buf || !len) return fail(STRO_ERR_INVALID, "null argument");
    std::snprintf(buf, len, "%s", s->last_path);
    return STRO_OK;
}

int stro_sim_set_arithmetic(stro_sim* s, int32_t arith) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (arith != STRO_ARITH_REFERENCE && arith != STRO_ARITH_FUSED)
        return fail(STRO_ERR_INVALID, "arithmetic must be STRO_ARITH_REFERENCE or STRO_ARITH_FUSED");
    s->arith = arith;
    return STRO_OK;
}

int stro_sim_get_arithmetic(stro_sim* s, int32_t* arith) {
    if (!s || !arith) return fail(STRO_ERR_INVALID, "null argument");
    *arith = s->arith;
    return STRO_OK;
}

int stro_sim_set_rows_tile(stro_sim* s, int32_t threads, int32_t rows) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (threads < 32 || threads > 256 || threads % 32 != 0 || rows < 1 || rows > 8)
        return fail(STRO_ERR_INVALID, "rows tile: threads a multiple of 32 up to 256, 1 to 8 rows");
    s->rows_threads = threads;
    s->rows_per_tile = rows;
    return STRO_OK;
}

int stro_sim_get_rows_tile(stro_sim* s, int32_t* threads, int32_t* rows) {
    if (!s || !threads || !rows) return fail(STRO_ERR_INVALID, "null argument");
    *threads = s->rows_threads;
    *rows = s->rows_per_tile;
    return STRO_OK;
}

int stro_sim_get_variant(stro_sim* s, int32_t* variant) {
    if (!s || !variant) return fail(STRO_ERR_INVALID, "null argument");
    *variant = s->variant;
    return STRO_OK;
}

int stro_sim_get_block(stro_sim* s, int32_t* bx, int32_t* by) {
    if (!s || !bx || !by) return fail(STRO_ERR_INVALID, "null argument");
    *bx = int32_t(s->block.x);
    *by = int32_t(s->block.y);
    return STRO_OK;
}

int stro_sim_autotune(stro_sim* s, int64_t steps, int32_t* bx, int32_t* by, double* glups) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (steps < 2) steps = 2;
    steps &= ~int64_t(1);
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    const size_t bytes = 19 * s->plane * s->esize;
    void* saved = nullptr;
    STRO_CUDA(cudaMalloc(&saved, bytes));
    cudaError_t e = cudaMemcpyAsync(saved, s->d_f, bytes, cudaMemcpyDeviceToDevice, st);
    double best = 1e300;
    dim3 best_shape = s->block;
    int best_variant = 0;
    int rc = e == cudaSuccess ? STRO_OK : cuda_fail(e, "autotune save");
    const int half = s->precision == STRO_FP16S ? 1 : 0;
    const bool saved_split = s->split;
    bool best_split = saved_split;
    const int geo = geo_on(s) ? 1 : 0;
    for (int split : {1, 0}) {
        if (!split && !geo) break;  // the split only exists for walled lattices
        s->split = split != 0;
        for (int variant : {0, 1, 2, 3}) {
            const dim3* shapes = variant == 2 ? kRowShapes : kShapes;
            const size_t nshapes = variant == 2 ? sizeof(kRowShapes) / sizeof(dim3)
                                                : sizeof(kShapes) / sizeof(dim3);
            for (size_t q = 0; q < nshapes && rc == STRO_OK; ++q) {
                const dim3 c = shapes[q];
                if ((variant == 0 || variant == 3) && c.x > 32 &&
                    int(c.x) > ((s->nx + 31) / 32) * 32)
                    continue;
                if (variant == 3 && (geo || c.x * c.y > 128)) continue;
                if (variant == 1 && !exact::kPair.supported(half, geo, false, s->nx, s->plane, c))
                    continue;
                if (variant == 2 && !exact::kRows.supported(half, geo, false, s->nx, s->ny,
                                                            int(c.x), int(c.y)))
                    continue;
                if (variant != 0 && split == 0) continue;  // the split only changes variant 0
                double sec = 0.0;
                rc = tune_sim_shape(s, steps, variant, c, &sec);
                if (rc == STRO_OK && sec < best) {
                    best = sec;
                    best_shape = c;
                    best_variant = variant;
                    best_split = s->split;
                }
            }
        }
    }
    s->split = best_split;
    e = cudaMemcpyAsync(s->d_f, saved, bytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(saved);
    if (rc != STRO_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "autotune restore");
    s->variant = best_variant;
    if (best_variant == 1) s->pair_block = best_shape;
    else if (best_variant == 2) {
        s->rows_threads = int(best_shape.x);
        s->rows_per_tile = int(best_shape.y);
    } else {
        s->block = best_shape;
    }
    if (bx) *bx = int32_t(best_shape.x);
    if (by) *by = int32_t(best_shape.y);
    if (glups) *glups = double(s->N) * double(steps) / best / 1e9;
    return STRO_OK;
}

int stro_batch_autotune(stro_batch* b, int64_t rounds, int32_t* mode, int32_t* bx, int32_t* by,
                        double* seconds) {
    if (!b) return fail(STRO_ERR_INVALID, "null batch");
    if (rounds < 2) rounds = 2;
    rounds &= ~int64_t(1);
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = b->ctx->stream;
    // save every state and step counter; the tuning runs are undone afterwards
    std::vector<void*> saved(b->sims.size(), nullptr);
    std::vector<int64_t> t0(b->sims.size());
    int rc = STRO_OK;
    for (size_t i = 0; i < b->sims.size() && rc == STRO_OK; ++i) {
        stro_sim* s = b->sims[i];
        const size_t bytes = 19 * s->plane * s->esize;
        t0[i] = s->steps_done;
        cudaError_t e = cudaMalloc(&saved[i], bytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(saved[i], s->d_f, bytes, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch autotune save");
    }
    const int old_mode = b->mode;
    const dim3 old_block = b->block;
    const double old_sec = b->gpu_seconds;
    double best = 1e300;
    int best_mode = old_mode;
    dim3 best_block = old_block;
    std::vector<int64_t> steps(b->sims.size(), rounds);
    for (int m : {int(STRO_BATCH_PERSISTENT), int(STRO_BATCH_ROUNDS)}) {
        for (const dim3& c : kShapes) {
            if (rc != STRO_OK) break;
            b->mode = m;
            b->block = c;
            for (size_t i = 0; i < b->sims.size(); ++i) b->sims[i]->steps_done = t0[i];
            const double g0 = b->gpu_seconds;
            rc = stro_batch_run(b, steps.data(), nullptr, nullptr, 0, nullptr);
            if (rc != STRO_OK) break;
            const double sec = b->gpu_seconds - g0;
            if (sec < best) {
                best = sec;
                best_mode = m;
                best_block = c;
            }
        }
    }
    for (size_t i = 0; i < b->sims.size(); ++i) {
        stro_sim* s = b->sims[i];
        if (saved[i]) {
            cudaMemcpyAsync(s->d_f, saved[i], 19 * s->plane * s->esize, cudaMemcpyDeviceToDevice, st);
        }
        s->steps_done = t0[i];
    }
    cudaStreamSynchronize(st);
    for (void* p : saved) cudaFree(p);
    drop_graph(b);
    b->gpu_seconds = old_sec;
    if (rc != STRO_OK) {
        b->mode = old_mode;
        b->block = old_block;
        return rc;
    }
    b->mode = best_mode;
    b->block = best_block;
    if (mode) *mode = best_mode;
    if (bx) *bx = int32_t(best_block.x);
    if (by) *by = int32_t(best_block.y);
    if (seconds) *seconds = best;
    return STRO_OK;
}

}  // extern "C"
