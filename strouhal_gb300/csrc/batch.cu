// Host side of batched stepping (C ABI stro_batch_*) and the launch-shape
// autotuners.
//
// A batch groups existing simulations of one precision on one context. A run
// advances instance i by steps[i] lattice steps, exactly as calling
// stro_sim_run on each in turn would (bitwise identical DDFs), in one of:
//   STRO_BATCH_PERSISTENT  one cooperative persistent kernel with a bounded
//                          grid barrier between rounds, captured in a CUDA
//                          graph together with the reset of its control word;
//   STRO_BATCH_ROUNDS      a CUDA graph of one launch per round;
//   STRO_BATCH_STREAMS     each instance's own launches on a stream of its
//                          own, enqueued in turns from this thread;
//   STRO_BATCH_SEQUENTIAL  the reference's order: one instance after another
//                          (the baseline the batch is measured against).
// The instantiated graph is cached and replayed while the schedule (step
// counts, logging, tile shape) is unchanged; the per-instance descriptors are
// re-uploaded before every replay.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
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
    double* d_fpart = nullptr;
    size_t fpart_cap = 0;
    double* d_samples = nullptr;
    size_t samples_cap = 0;
    std::vector<cudaStream_t> streams;  // STRO_BATCH_STREAMS: one per instance
    uint32_t* d_tiles = nullptr;  // rounds mode: bulk tile list, then boundary tile list
    size_t tiles_cap = 0;
    uint16_t* d_tile_inst = nullptr;  // instance of every tile
    size_t tile_inst_cap = 0;
    int split = 1;
    int64_t last_bulk = 0, last_edge = 0;
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

// Rounds-mode runs longer than this are launched round by round on the
// stream instead of being captured into one graph (a graph node per round).
constexpr int64_t kMaxGraphRounds = 32768;

// One instance's force-probe schedule in a sampled run (Ladder.measure): the
// first probe at round `first` (an odd step), then every `period` rounds,
// `count` probes, each over the box {x0, x1, y0, y1}.
struct SamplePlan {
    int64_t first = -1;
    int32_t period = 0;
    int32_t count = 0;
    int box[4] = {0, 0, 0, 0};
};

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

// STRO_BATCH_STREAMS: each instance on a stream of its own, every instance's
// work enqueued from this thread before any is waited for. Each instance runs
// exactly what stro_sim_run would (its own tuned kernels, CUDA graphs of its
// plain steps) and the GPU overlaps the instances, which small lattices leave
// room for. The instance streams wait for the batch event ev0 (recorded on
// the context stream by the caller) and the context stream waits for each
// instance's last event, so ev0 / ev1 on the context stream bracket the run.
int ensure_streams(stro_batch* b) {
    while (b->streams.size() < b->sims.size()) {
        cudaStream_t x = nullptr;
        STRO_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        b->streams.push_back(x);
    }
    return STRO_OK;
}

// Graph length for a run of `count` plain steps that repeats: the whole run
// when it is short, else runs of kRunGraphSteps.
int64_t repeat_graph_steps(int64_t count) {
    if (count >= 2 && count <= 256 && count % 2 == 0) return count;
    return count >= 2 * kRunGraphSteps ? kRunGraphSteps : 0;
}

int run_streams(stro_batch* b, const int64_t* steps, const int32_t* log_every,
                std::vector<std::vector<double>>& traces) {
    const size_t n = b->sims.size();
    int rc = ensure_streams(b);
    if (rc != STRO_OK) return rc;
    std::vector<size_t> off(n, 0), cnt(n, 0);
    size_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        const int64_t le = log_every ? log_every[i] : 0;
        if (le > 0) {
            cnt[i] = size_t(1 + steps[i] / le);
            off[i] = total;
            total += cnt[i];
        }
    }
    rc = grow(&b->d_traces, &b->traces_cap, total);
    if (rc != STRO_OK) return rc;
    // per instance: next step, steps left, trace slots written
    struct Cursor {
        int64_t t = 0, left = 0;
        size_t k = 0;
        bool done = false;
    };
    std::vector<Cursor> cur(n);
    size_t queued = 0;
    for (size_t i = 0; i < n && rc == STRO_OK; ++i) {
        stro_sim* s = b->sims[i];
        cudaError_t e = cudaStreamWaitEvent(b->streams[i], b->ev0, 0);
        if (e == cudaSuccess) e = cudaEventRecord(s->ev0, b->streams[i]);
        if (e != cudaSuccess) rc = cuda_fail(e, "instance stream");
        cur[i].t = s->steps_done;
        cur[i].left = steps[i];
        queued = i + 1;
    }
    // One piece of each instance in turn (a logging interval, or up to 1024
    // steps): a stream's queue of pending launches is bounded, and a host
    // thread blocked on one full queue must not leave the others without work.
    for (bool more = true; more && rc == STRO_OK;) {
        more = false;
        for (size_t i = 0; i < n && rc == STRO_OK; ++i) {
            Cursor& c = cur[i];
            if (c.done) continue;
            stro_sim* s = b->sims[i];
            cudaStream_t ss = b->streams[i];
            const int64_t le = log_every ? log_every[i] : 0;
            s->stream = ss;
            auto log = [&]() {  // sum |u|^2 into trace slot k, as observables() computes it
                cudaError_t e = launch_observables(field_view(s), s->precision == STRO_FP16S,
                                                   s->omega, s->d_partials, s->d_out, ss);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(b->d_traces + off[i] + c.k, s->d_out, sizeof(double),
                                        cudaMemcpyDeviceToDevice, ss);
                ++c.k;
                return e == cudaSuccess ? STRO_OK : cuda_fail(e, "instance trace");
            };
            if (le > 0 && c.k == 0) {
                rc = log();
            } else if (le > 0 && c.left >= le) {
                rc = launch_plain_steps(s, c.t, le, repeat_graph_steps(le));
                c.t += le;
                c.left -= le;
                if (rc == STRO_OK) rc = log();
            } else if (c.left > 0) {
                const int64_t piece = le > 0 ? c.left : std::min<int64_t>(c.left, 1024);
                rc = launch_plain_steps(s, c.t, piece,
                                        piece >= 2 * kRunGraphSteps ? kRunGraphSteps : 0);
                c.t += piece;
                c.left -= piece;
            }
            if (rc == STRO_OK && c.left == 0 && (le == 0 || c.k > 0)) {
                cudaError_t e = cudaEventRecord(s->ev1, ss);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(b->ctx->stream, s->ev1, 0);
                if (e != cudaSuccess) rc = cuda_fail(e, "instance stream");
                c.done = true;
            }
            s->stream = nullptr;
            more = more || !c.done;
        }
    }
    // wait for every instance that was enqueued, whatever happened after it
    for (size_t i = 0; i < queued; ++i) {
        cudaError_t e = cudaStreamSynchronize(b->streams[i]);
        if (e != cudaSuccess && rc == STRO_OK) rc = cuda_fail(e, "instance stream");
    }
    if (rc != STRO_OK) return rc;
    for (size_t i = 0; i < n; ++i) {
        stro_sim* s = b->sims[i];
        float ms = 0.0f;
        STRO_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        s->gpu_seconds += double(ms) * 1e-3;
        s->steps_done += steps[i];
        const int re = check_rows_error(s);
        if (re != STRO_OK) return re;
        if (cnt[i]) {
            traces[i].resize(cnt[i]);
            STRO_CUDA(cudaMemcpy(traces[i].data(), b->d_traces + off[i], cnt[i] * sizeof(double),
                                 cudaMemcpyDeviceToHost));
        }
    }
    return STRO_OK;
}

// A lattice whose geometry has walls, inlets, outlets or solid fractions
// (some cell flag or geometry word set); its batch tiles are 2-D blocks.
bool walled(const stro_sim* s) {
    if (s->cell_host.size() != s->N || s->geo_host.size() != s->N) return false;
    for (size_t c = 0; c < s->N; ++c)
        if (s->cell_host[c] != 0 || s->geo_host[c] != 0) return true;
    return false;
}

int run_fused(stro_batch* b, const int64_t* steps, const int32_t* log_every,
              std::vector<std::vector<double>>& traces, const SamplePlan* plans = nullptr,
              std::vector<std::vector<double>>* samples = nullptr) {
    const size_t n = b->sims.size();
    cudaStream_t st = b->ctx->stream;
    const int geo = batch_geo(b) ? 1 : 0;
    const int feat = batch_feat(b);
    int probes = 0;
    if (plans && geo)
        for (size_t i = 0; i < n; ++i) probes |= plans[i].count > 0 ? 1 : 0;
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
    std::vector<size_t> ramp_off(n, size_t(-1)), trace_off(n, 0), sample_off(n, 0);
    size_t tiles = 0, trace_total = 0, sample_total = 0;
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
        division_magic(uint32_t(s->nx), &I.div_nx_m, &I.div_nx_s);
        division_magic(uint32_t(s->ny), &I.div_ny_m, &I.div_ny_s);
        I.ntiles = (I.cells + threads - 1) / threads;
        if (walled(s)) {
            I.tiles_x = (uint32_t(s->nx) + b->block.x - 1) / b->block.x;
            I.tiles_y = (uint32_t(s->ny) + b->block.y - 1) / b->block.y;
            I.ntiles = I.tiles_x * I.tiles_y * uint32_t(s->nz);
        }
        I.tile_begin = uint32_t(tiles);
        tiles += I.ntiles;
        if (I.log_every > 0) {
            I.trace_cap = int32_t((I.steps + I.log_every - 1) / I.log_every);
            trace_off[k] = trace_total;
            trace_total += size_t(I.trace_cap);
        }
        I.probe_first = -1;
        if (probes && plans[order[k]].count > 0) {
            const SamplePlan& pl = plans[order[k]];
            I.probe_first = pl.first;
            I.probe_period = pl.period;
            I.probe_count = pl.count;
            I.a.box_x0 = pl.box[0];
            I.a.box_x1 = pl.box[1];
            I.a.box_y0 = pl.box[2];
            I.a.box_y1 = pl.box[3];
            sample_off[k] = sample_total;
            sample_total += 3 * size_t(pl.count);
        }
        max_steps = std::max(max_steps, I.steps);
    }
    if (tiles >= (1ull << 31)) return fail(STRO_ERR_INVALID, "batch too large");
    std::vector<uint16_t> tile_inst(tiles);
    for (size_t k = 0; k < n; ++k)
        std::fill(tile_inst.begin() + inst[k].tile_begin,
                  tile_inst.begin() + inst[k].tile_begin + inst[k].ntiles, uint16_t(k));
    // Rounds mode on a walled batch: bulk tiles (every cell fluid, without
    // wall neighbours or solid fraction) go to the wall-free kernels, the rest
    // to the wall-aware ones. Both lists are in instance order, so the tiles of
    // the instances still running at round r are a prefix of each.
    const bool split = b->mode == STRO_BATCH_ROUNDS && geo && b->split;
    std::vector<uint32_t> tile_list;
    std::vector<uint32_t> bulk_end(n, 0), edge_end(n, 0);
    uint32_t nbulk_total = 0;
    if (split) {
        std::vector<uint32_t> edges, bulk_k, edge_k;
        tile_list.reserve(tiles);
        for (size_t k = 0; k < n; ++k) {
            const stro_sim* s = b->sims[order[k]];
            if (inst[k].tiles_x != 0) {
                block_lists(s, b->block, bulk_k, edge_k);
                for (uint32_t t : bulk_k) tile_list.push_back(inst[k].tile_begin + t);
                for (uint32_t t : edge_k) edges.push_back(inst[k].tile_begin + t);
            } else {  // no walls: every tile is bulk
                for (uint32_t t = 0; t < inst[k].ntiles; ++t)
                    tile_list.push_back(inst[k].tile_begin + t);
            }
            bulk_end[k] = uint32_t(tile_list.size());
            edge_end[k] = uint32_t(edges.size());
        }
        nbulk_total = uint32_t(tile_list.size());
        tile_list.insert(tile_list.end(), edges.begin(), edges.end());
    }
    int rc = grow(&b->d_inst, &b->inst_cap, n);
    if (rc == STRO_OK) rc = grow(&b->d_kepart, &b->kepart_cap, tiles);
    if (rc == STRO_OK) rc = grow(&b->d_ramp, &b->ramp_cap, ramp.size());
    if (rc == STRO_OK) rc = grow(&b->d_traces, &b->traces_cap, trace_total);
    if (rc == STRO_OK && probes) rc = grow(&b->d_fpart, &b->fpart_cap, 3 * tiles);
    if (rc == STRO_OK && probes) rc = grow(&b->d_samples, &b->samples_cap, sample_total);
    if (rc == STRO_OK && split) rc = grow(&b->d_tiles, &b->tiles_cap, tile_list.size());
    if (rc == STRO_OK) rc = grow(&b->d_tile_inst, &b->tile_inst_cap, tiles);
    if (rc == STRO_OK && !b->d_ctl) STRO_CUDA(cudaMalloc(&b->d_ctl, sizeof(BatchCtl)));
    if (rc != STRO_OK) return rc;
    for (size_t k = 0; k < n; ++k) {
        inst[k].ramp = ramp_off[k] == size_t(-1) ? nullptr : b->d_ramp + ramp_off[k];
        inst[k].trace = inst[k].log_every > 0 ? b->d_traces + trace_off[k] : nullptr;
        inst[k].samples = inst[k].probe_first >= 0 ? b->d_samples + sample_off[k] : nullptr;
    }
    STRO_CUDA(cudaMemcpyAsync(b->d_inst, inst.data(), n * sizeof(BatchInstance),
                              cudaMemcpyHostToDevice, st));
    if (!ramp.empty())
        STRO_CUDA(cudaMemcpyAsync(b->d_ramp, ramp.data(), ramp.size() * sizeof(float),
                                  cudaMemcpyHostToDevice, st));
    if (split)
        STRO_CUDA(cudaMemcpyAsync(b->d_tiles, tile_list.data(), tile_list.size() * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, st));
    STRO_CUDA(cudaMemcpyAsync(b->d_tile_inst, tile_inst.data(), tiles * sizeof(uint16_t),
                              cudaMemcpyHostToDevice, st));
    b->last_bulk = split ? nbulk_total : 0;
    b->last_edge = split ? int64_t(tile_list.size()) - nbulk_total : 0;
    BatchArgs args{};
    args.inst = b->d_inst;
    args.tile_inst = b->d_tile_inst;
    args.count = int32_t(n);
    args.max_steps = max_steps;
    args.kepart = b->d_kepart;
    args.fpart = probes ? b->d_fpart : nullptr;
    args.ctl = b->d_ctl;
    args.spin_limit = b->spin_limit;

    // schedule key of the cached graph
    std::vector<int64_t> key = {b->mode, int64_t(b->block.x), int64_t(b->block.y), geo, feat,
                                b->half, int64_t(n), max_steps, int64_t(tiles),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_inst)),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_kepart)),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_ctl)), probes,
                                int64_t(reinterpret_cast<uintptr_t>(args.fpart)), split,
                                int64_t(reinterpret_cast<uintptr_t>(b->d_tiles)),
                                int64_t(reinterpret_cast<uintptr_t>(b->d_tile_inst))};
    for (size_t k = 0; k < n; ++k) {
        key.push_back(bulk_end[k]);
        key.push_back(edge_end[k]);
        key.push_back(inst[k].steps);
        key.push_back(inst[k].log_every);
        key.push_back(inst[k].ntiles);
        key.push_back(inst[k].t0 & 1);
        key.push_back(inst[k].probe_first);
        key.push_back(inst[k].probe_period);
        key.push_back(inst[k].probe_count);
    }
    // what round r launches in rounds mode: the active tile prefix, and whether
    // some instance logs or probes in it
    auto round_plan = [&](int64_t r, uint32_t* active, uint32_t* nbulk, uint32_t* nedge,
                          bool* logs, bool* probing) {
        *active = *nbulk = *nedge = 0;
        *logs = *probing = false;
        for (size_t k = 0; k < n; ++k) {
            if (inst[k].steps <= r) break;
            *active = inst[k].tile_begin + inst[k].ntiles;
            *nbulk = bulk_end[k];
            *nedge = edge_end[k];
            if (inst[k].log_every > 0 && r % inst[k].log_every == 0 && ((inst[k].t0 + r) & 1) == 0)
                *logs = true;
            if (inst[k].probe_first >= 0 && r >= inst[k].probe_first &&
                (r - inst[k].probe_first) % inst[k].probe_period == 0 &&
                (r - inst[k].probe_first) / inst[k].probe_period < inst[k].probe_count)
                *probing = true;
        }
    };
    auto launch_rounds = [&]() {
        cudaError_t le = cudaSuccess;
        for (int64_t r = 0; r < max_steps && le == cudaSuccess; ++r) {
            uint32_t active, nbulk, nedge;
            bool logs, probing;
            round_plan(r, &active, &nbulk, &nedge, &logs, &probing);
            if (split)
                le = launch_batch_round_lists(args, b->half, feat, probing ? 1 : 0, r, b->d_tiles,
                                              nbulk, b->d_tiles + nbulk_total, nedge, b->block, st);
            else
                le = launch_batch_round(args, b->half, geo, feat, probing ? 1 : 0, r, active,
                                        b->block, st);
            if (le == cudaSuccess && (logs || probing)) le = launch_batch_fold(args, r, st);
        }
        return le;
    };
    const bool stream_rounds = b->mode == STRO_BATCH_ROUNDS && max_steps > kMaxGraphRounds;
    unsigned grid = 0;
    if (b->mode == STRO_BATCH_PERSISTENT) {
        const int per_sm = batch_persistent_blocks_per_sm(b->half, geo, feat, probes, b->block);
        if (per_sm <= 0) return fail(STRO_ERR_CUDA, "persistent kernel cannot be resident");
        grid = unsigned(std::min<size_t>(tiles, size_t(per_sm) * b->ctx->sm_count));
        if (grid == 0) grid = 1;
        key.push_back(grid);
    }
    if (stream_rounds) {
        drop_graph(b);
        STRO_CUDA(launch_rounds());
        b->last_path = "rounds-stream";
    } else if (key != b->exec_key) {
        drop_graph(b);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
        cudaError_t le = cudaSuccess;
        if (b->mode == STRO_BATCH_PERSISTENT) {
            le = cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchCtl), st);
            if (le == cudaSuccess)
                le = launch_batch_persistent(args, b->half, geo, feat, probes, grid, b->block, st);
        } else {
            le = launch_rounds();
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
    if (!stream_rounds) {
        b->last_path = b->mode == STRO_BATCH_PERSISTENT ? "persistent-graph" : "rounds-graph";
        STRO_CUDA(cudaGraphLaunch(b->exec, st));
    }
    b->last_rounds = max_steps;
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
    if (samples) {
        std::vector<double> hs(sample_total);
        if (sample_total)
            STRO_CUDA(cudaMemcpy(hs.data(), b->d_samples, sample_total * sizeof(double),
                                 cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < n; ++k) {
            const size_t i = order[k];
            const size_t cnt = plans ? 3 * size_t(std::max(plans[i].count, 0)) : 0;
            if (inst[k].probe_first >= 0)
                (*samples)[i].assign(hs.begin() + sample_off[k], hs.begin() + sample_off[k] + cnt);
            else
                (*samples)[i].assign(cnt, 0.0);  // no geometry: no momentum exchange
        }
    }
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
    if (e == cudaSuccess && variant == 2) {
        e = cudaMemcpyAsync(&err, s->d_error, sizeof err, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    s->block = saved;
    s->pair_block = saved_pair;
    s->variant = saved_variant;
    s->rows_threads = saved_rows;
    s->rows_per_tile = saved_tile;
    s->gpu_seconds = g0;
    if (e != cudaSuccess) return cuda_fail(e, "autotune launch");
    if (err != 0) {
        cudaMemsetAsync(s->d_error, 0, sizeof(int), st);
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
    if (count > 65535) return fail(STRO_ERR_INVALID, "a batch holds at most 65535 lattices");
    *out = nullptr;
    for (int32_t i = 0; i < count; ++i) {
        if (!sims[i]) return fail(STRO_ERR_INVALID, "null simulation in batch");
        if (sims[i]->ctx != ctx) return fail(STRO_ERR_INVALID, "batch spans contexts");
        if (sims[i]->precision != sims[0]->precision)
            return fail(STRO_ERR_INVALID, "batch mixes precisions");
        if (sims[i]->arith != STRO_ARITH_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference arithmetic only");
        if (sims[i]->collision != STRO_COLLISION_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference collision only");
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
    cudaFree(b->d_fpart);
    cudaFree(b->d_samples);
    cudaFree(b->d_tiles);
    cudaFree(b->d_tile_inst);
    for (cudaStream_t x : b->streams) cudaStreamDestroy(x);
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
    if (mode != STRO_BATCH_PERSISTENT && mode != STRO_BATCH_ROUNDS && mode != STRO_BATCH_SEQUENTIAL &&
        mode != STRO_BATCH_STREAMS)
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

int stro_batch_set_split(stro_batch* b, int32_t on) {
    if (!b) return fail(STRO_ERR_INVALID, "null batch");
    b->split = on ? 1 : 0;
    return STRO_OK;
}

int stro_batch_split_tiles(const stro_batch* b, int64_t* bulk, int64_t* edge) {
    if (!b || !bulk || !edge) return fail(STRO_ERR_INVALID, "null argument");
    *bulk = b->last_bulk;
    *edge = b->last_edge;
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
        if (b->sims[i]->collision != STRO_COLLISION_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference collision only");
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
    } else if (b->mode == STRO_BATCH_STREAMS) {
        rc = run_streams(b, steps, log_every, tr);
        b->last_path = "streams";
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

int stro_batch_run_sampled(stro_batch* b, const int64_t* transient, const int64_t* sample_steps,
                           const int64_t* stride, const int32_t* boxes, double* const* forces,
                           const int64_t* capacity, int64_t* samples) {
    if (!b || !transient || !sample_steps || !stride || !boxes || !forces || !capacity || !samples)
        return fail(STRO_ERR_INVALID, "null argument");
    const size_t n = b->sims.size();
    std::vector<SamplePlan> plans(n);
    std::vector<int64_t> steps(n);
    bool short_buffer = false;
    for (size_t i = 0; i < n; ++i) {
        stro_sim* s = b->sims[i];
        const int32_t* bx = boxes + 4 * i;
        if (s->arith != STRO_ARITH_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference arithmetic only");
        if (s->collision != STRO_COLLISION_REFERENCE)
            return fail(STRO_ERR_INVALID, "batches run the reference collision only");
        if (!s->wants_forces) return fail(STRO_ERR_STATE, "force samples require wants_forces");
        if (s->steps_done % 2 != 0)
            return fail(STRO_ERR_STATE, "a sampled run must start at an even step count");
        if (transient[i] < 0 || sample_steps[i] < 0 || stride[i] < 1)
            return fail(STRO_ERR_INVALID, "negative step counts or stride < 1");
        if (bx[0] < 0 || bx[1] >= s->nx || bx[2] < 0 || bx[3] >= s->ny || bx[0] > bx[1] ||
            bx[2] > bx[3])
            return fail(STRO_ERR_INVALID, "force box outside the lattice");
        // the schedule of stro_sim_run_sampled (Ladder.swift:55-66)
        const int64_t T = transient[i] & ~int64_t(1);
        const int64_t chunk = std::max<int64_t>(2, stride[i] - 2) & ~int64_t(1);
        const int64_t cnt = (sample_steps[i] + chunk + 1) / (chunk + 2);
        if (chunk + 2 > INT32_MAX || cnt > INT32_MAX)
            return fail(STRO_ERR_INVALID, "stride or sample count too large");
        samples[i] = cnt;
        if (cnt > capacity[i] || (cnt > 0 && !forces[i])) short_buffer = true;
        plans[i].first = cnt > 0 ? T + chunk + 1 : -1;
        plans[i].period = int32_t(chunk + 2);
        plans[i].count = int32_t(cnt);
        std::copy(bx, bx + 4, plans[i].box);
        steps[i] = T + cnt * (chunk + 2);
    }
    if (short_buffer) return fail(STRO_ERR_INVALID, "a sample buffer is smaller than its run");
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = b->ctx->stream;
    if (b->mode == STRO_BATCH_SEQUENTIAL) {  // the reference's order, variant after variant
        const double g0 = b->gpu_seconds;
        double g = 0.0;
        for (size_t i = 0; i < n; ++i) {
            stro_sim* s = b->sims[i];
            const double s0 = s->gpu_seconds;
            int64_t got = 0;
            const int rc = stro_sim_run_sampled(s, transient[i], sample_steps[i], stride[i],
                                                boxes[4 * i], boxes[4 * i + 1], boxes[4 * i + 2],
                                                boxes[4 * i + 3], forces[i], capacity[i], &got,
                                                nullptr);
            if (rc != STRO_OK) return rc;
            g += s->gpu_seconds - s0;
        }
        b->gpu_seconds = g0 + g;
        b->last_path = "sequential";
        return STRO_OK;
    }
    if (b->mode == STRO_BATCH_STREAMS) {  // stro_sim_run_sampled on every instance at once
        int rc = ensure_streams(b);
        if (rc != STRO_OK) return rc;
        STRO_CUDA(cudaEventRecord(b->ev0, st));
        std::vector<SampledRun> runs(n);
        size_t queued = 0;
        for (size_t i = 0; i < n && rc == STRO_OK; ++i) {
            stro_sim* s = b->sims[i];
            const cudaError_t e = cudaStreamWaitEvent(b->streams[i], b->ev0, 0);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "instance stream");
                break;
            }
            s->stream = b->streams[i];
            int64_t got = 0;
            rc = sampled_begin(s, transient[i], sample_steps[i], stride[i], boxes + 4 * i,
                               forces[i], capacity[i], &got, nullptr, &runs[i]);
            s->stream = nullptr;
            if (rc != STRO_OK) break;
            queued = i + 1;
        }
        // Enqueue the schedules in turns, one piece of each instance at a
        // time: a stream's queue of pending launches is bounded, and a host
        // thread blocked on one full queue must not leave the other streams
        // without work.
        for (bool more = true; more && rc == STRO_OK;) {
            more = false;
            for (size_t i = 0; i < n && rc == STRO_OK; ++i) {
                if (runs[i].done) continue;
                b->sims[i]->stream = b->streams[i];
                rc = sampled_advance(b->sims[i], &runs[i]);
                b->sims[i]->stream = nullptr;
                more = more || !runs[i].done;
            }
        }
        for (size_t i = 0; i < n && rc == STRO_OK; ++i) {
            const cudaError_t w = cudaStreamWaitEvent(st, b->sims[i]->ev1, 0);
            if (w != cudaSuccess) rc = cuda_fail(w, "instance stream");
        }
        if (rc == STRO_OK) {
            const cudaError_t e = cudaEventRecord(b->ev1, st);
            if (e != cudaSuccess) rc = cuda_fail(e, "batch event");
        }
        for (size_t i = 0; i < queued; ++i) {  // every enqueued run is waited for and freed
            b->sims[i]->stream = b->streams[i];
            const int r = sampled_finish(b->sims[i], &runs[i]);
            b->sims[i]->stream = nullptr;
            if (rc == STRO_OK) rc = r;
        }
        if (rc != STRO_OK) return rc;
        STRO_CUDA(cudaEventSynchronize(b->ev1));
        float ms = 0.0f;
        STRO_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        b->gpu_seconds += double(ms) * 1e-3;
        b->last_path = "streams";
        return STRO_OK;
    }
    std::vector<std::vector<double>> tr(n), out(n);
    STRO_CUDA(cudaEventRecord(b->ev0, st));
    const int rc = run_fused(b, steps.data(), nullptr, tr, plans.data(), &out);
    if (rc != STRO_OK) return rc;
    STRO_CUDA(cudaEventRecord(b->ev1, st));
    STRO_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.0f;
    STRO_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->gpu_seconds += double(ms) * 1e-3;
    for (size_t i = 0; i < n; ++i)
        if (!out[i].empty()) std::copy(out[i].begin(), out[i].end(), forces[i]);
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
    if (variant < 0 || variant > 5) return fail(STRO_ERR_INVALID, "variant must be 0..5");
    s->variant = variant;
    return STRO_OK;
}

int stro_sim_set_block_split(stro_sim* s, int32_t enabled) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (enabled < 0 || enabled > 5) return fail(STRO_ERR_INVALID, "split must be 0 to 5");
    s->split = enabled != 0;
    s->edge_colmajor = enabled == 2;
    s->face_lists = enabled != 3;
    s->merged_faces = enabled == 4;
    s->pair_bulk = enabled == 5;
    return STRO_OK;
}

int stro_sim_set_graphs(stro_sim* s, int32_t enabled) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    s->graphs = enabled != 0;
    if (!s->graphs) drop_graphs(s);
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

int stro_sim_split_blocks(const stro_sim* s, int64_t* bulk, int64_t* face, int64_t* edge) {
    if (!s || !bulk || !face || !edge) return fail(STRO_ERR_INVALID, "null argument");
    *bulk = s->nbulk;
    *face = s->nface;
    *edge = s->nedge;
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

int stro_sim_set_collision(stro_sim* s, int32_t collision) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (collision != STRO_COLLISION_REFERENCE && collision != STRO_COLLISION_KBC)
        return fail(STRO_ERR_INVALID, "collision must be STRO_COLLISION_REFERENCE or STRO_COLLISION_KBC");
    if (collision == STRO_COLLISION_KBC) {
        if (s->c_smago > 0.0f)
            return fail(STRO_ERR_INVALID, "the KBC collision has no Smagorinsky model");
        for (float e : s->eps)
            if (e > 0.0f)
                return fail(STRO_ERR_INVALID, "the KBC collision has no partially solid cells");
    }
    s->collision = collision;
    return STRO_OK;
}

int stro_sim_get_collision(stro_sim* s, int32_t* collision) {
    if (!s || !collision) return fail(STRO_ERR_INVALID, "null argument");
    *collision = s->collision;
    return STRO_OK;
}

int stro_sim_set_outflow_mode(stro_sim* s, int32_t mode) {
    if (!s) return fail(STRO_ERR_INVALID, "null simulation handle");
    if (mode != STRO_OUTFLOW_DORMANT && mode != STRO_OUTFLOW_PRESSURE)
        return fail(STRO_ERR_INVALID, "outflow mode must be STRO_OUTFLOW_DORMANT or STRO_OUTFLOW_PRESSURE");
    s->outflow = mode;
    return STRO_OK;
}

int stro_sim_get_outflow_mode(stro_sim* s, int32_t* mode) {
    if (!s || !mode) return fail(STRO_ERR_INVALID, "null argument");
    *mode = s->outflow;
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

int stro_sim_set_spin_limit(stro_sim* s, int64_t polls) {
    if (!s || polls < 0) return fail(STRO_ERR_INVALID, "bad spin limit");
    s->rows_polls = polls;
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
    bool best_col = s->edge_colmajor;
    bool best_face = s->face_lists;
    bool best_merged = s->merged_faces;
    bool best_pair = s->pair_bulk;
    const int geo = geo_on(s) ? 1 : 0;
    // split 2: the split with the boundary blocks' odd pass in column-major
    // order; 3: the split without x-face blocks; 4: bulk and x-face blocks in
    // one launch; 5: as 4 with FP16 bulk blocks two cells per thread
    for (int split : {1, 4, 5, 2, 3, 0}) {
        if (split != 1 && !geo) break;  // the split only exists for walled lattices
        if (split == 5 && (!half || s->collision != STRO_COLLISION_REFERENCE)) continue;
        s->split = split != 0;
        s->edge_colmajor = split == 2;
        s->face_lists = split != 3;
        s->merged_faces = split == 4;
        s->pair_bulk = split == 5;
        for (int variant : {0, 1, 2, 3, 4, 5}) {
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
                if ((variant == 4 || variant == 5) &&
                    !exact::kPair.wide_supported(half, geo, false, s->nx, s->ny, s->plane, c,
                                                 variant == 4 ? 4 : 8))
                    continue;
                if (variant == 2 && !exact::kRows.supported(half, geo, false, s->nx, s->ny,
                                                            int(c.x), int(c.y)))
                    continue;
                if (variant != 0 && split != 1) continue;  // the split only changes variant 0
                if (variant != 0 && s->collision != STRO_COLLISION_REFERENCE) continue;
                double sec = 0.0;
                rc = tune_sim_shape(s, steps, variant, c, &sec);
                if (rc == STRO_OK && sec < best) {
                    best = sec;
                    best_shape = c;
                    best_variant = variant;
                    best_split = s->split;
                    best_col = s->edge_colmajor;
                    best_face = s->face_lists;
                    best_merged = s->merged_faces;
                    best_pair = s->pair_bulk;
                }
            }
        }
    }
    s->split = best_split;
    s->edge_colmajor = best_col;
    s->face_lists = best_face;
    s->merged_faces = best_merged;
    s->pair_bulk = best_pair;
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
