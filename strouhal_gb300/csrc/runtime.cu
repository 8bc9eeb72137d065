// Host runtime of the C ABI (include/strouhal_c.h): the GB300 counterpart of
// the reference's GPU and Simulation classes (Sources/StrouhalCore/Sim.swift).
//
// Design (one process, one GPU):
//   - one CUDA stream per context; every call is stream-ordered and
//     synchronous at return, like Simulation.run's final wait (Sim.swift:326);
//   - DDFs live in HBM as 19 planes with a padded plane stride (multiple of 64
//     elements) so every plane starts 128-byte aligned; the canonical
//     unpadded layout only exists at the upload/download/digest boundary;
//   - geometry is precomputed once on the host (Sim.swift:227-255) and packed
//     into a cell byte (even pass) and a geometry word (odd pass);
//   - the per-step uniforms, including the cosine ramp (Sim.swift:258-281),
//     are computed on the host and passed by value to each launch;
//   - GPU time is accumulated from CUDA events around each run (gpuSeconds).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "runtime_internal.h"
#include "sha256.h"

using namespace stro;
using namespace stro::rt;

namespace {

thread_local std::string g_error;

constexpr int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
constexpr int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
constexpr int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};

uint64_t padded_plane(uint64_t N) { return (N + 63) / 64 * 64; }

}  // namespace

namespace stro {
namespace rt {

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? STRO_ERR_OOM : STRO_ERR_CUDA;
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

bool geo_on(const stro_sim* s) { return s->any_wall || s->has_eps; }

bool sponge_active(const stro_sim* s) {
    return s->sponge_on && s->sponge_x0 < float(s->nx - 1);
}
bool force_on(const stro_sim* s) {
    return (s->has_ffield && s->ffield_nonzero) || s->force[0] != 0.0f || s->force[1] != 0.0f ||
           s->force[2] != 0.0f;
}
int feat_on(const stro_sim* s) {
    if (s->collision == STRO_COLLISION_KBC) return 3;
    if (s->c_smago > 0.0f) return 2;  // features with the Smagorinsky block compiled in
    return (s->has_eps || sponge_active(s) || force_on(s)) ? 1 : 0;
}

dim3 default_block(int nx) {
    int bx = ((nx + 31) / 32) * 32;
    if (bx > 256) bx = 256;
    if (bx < 32) bx = 32;
    int by = 256 / bx;
    if (by < 1) by = 1;
    return dim3(bx, by, 1);
}

// Cosine ramp factor at step t, Sim.swift:258-266.
float ramp_factor(const stro_sim* s, int64_t t) {
    if (s->ramp_steps <= 0) return 1.0f;
    const double x = std::fmin(1.0, double(t) / double(s->ramp_steps));
    return 1.0f * float(0.5 * (1.0 - std::cos(3.141592653589793 * x)));
}

// Writes every field of *a (its padding is left as it was, so a zeroed object
// stays comparable byte for byte).
static void fill_step_args(const stro_sim* s, int64_t t, StepArgs* out) {
    StepArgs& a = *out;
    a.f = s->d_f;
    a.plane = s->plane;
    const bool fits = 19 * s->plane < (uint64_t(1) << 32);
    for (int i = 0; i < 19; ++i) a.poff[i] = fits ? uint32_t(uint64_t(i) * s->plane) : 0u;
    a.nx = s->nx; a.ny = s->ny; a.nz = s->nz;
    a.cell = s->d_cell;
    a.geo = s->d_geo;
    a.lmask = s->d_lmask;
    a.eps = s->d_eps;
    a.ffield = (s->has_ffield && s->ffield_nonzero) ? s->d_ffield : nullptr;
    a.ffield_plane = uint32_t(s->N);
    a.omega = s->omega;
    a.omega_minus = s->omega_minus;
    a.tau0 = 1.0f / s->omega;  // IEEE single division, as the kernels would do it
    const float r = ramp_factor(s, t);
    a.uin = s->uin * r;
    a.c_smago = s->c_smago;
    a.fx = s->force[0]; a.fy = s->force[1]; a.fz = s->force[2];
    a.ulid_x = s->lid[0] * r; a.ulid_y = s->lid[1] * r; a.ulid_z = s->lid[2] * r;
    a.inflow_uniform = s->inflow_uniform;
    if (s->sponge_on) {
        a.sponge_x0 = s->sponge_x0;
        a.sponge_inv_w = 1.0f / s->sponge_width;
        a.sponge_tau = s->sponge_tau;
    } else {
        a.sponge_x0 = 1e9f; a.sponge_inv_w = 0.0f; a.sponge_tau = 1.0f;
    }
    a.force_on = force_on(s) ? 1 : 0;
    a.outflow_pressure = s->outflow == STRO_OUTFLOW_PRESSURE ? 1 : 0;
    a.box_x0 = 0; a.box_x1 = -1; a.box_y0 = 0; a.box_y1 = -1;
    a.f_out = nullptr;
    a.partials = s->d_partials;
}

StepArgs step_args(const stro_sim* s, int64_t t) {
    StepArgs a;
    std::memset(&a, 0, sizeof a);
    fill_step_args(s, t, &a);
    return a;
}

FieldView field_view(const stro_sim* s) {
    FieldView v{};
    v.f = s->d_f;
    v.plane = s->plane;
    v.nx = uint32_t(s->nx); v.ny = uint32_t(s->ny); v.nz = uint32_t(s->nz);
    v.N = uint32_t(s->N);
    v.cell = geo_on(s) ? s->d_cell : nullptr;
    v.ffield = s->has_ffield ? s->d_ffield : nullptr;
    v.fx = s->force[0]; v.fy = s->force[1]; v.fz = s->force[2];
    return v;
}

// Neighbour masks (Sim.swift:227-255) and the packed device geometry.
int upload_geometry(stro_sim* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const uint64_t N = s->N;
    s->smask.assign(N, 0u);
    s->lmask.assign(N, 0u);
    s->any_wall = false;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const uint64_t idx = (uint64_t(z) * ny + y) * nx + x;
                const uint8_t c = s->flags[idx];
                if (c != STRO_FLUID) { s->any_wall = true; continue; }
                uint32_t sm = 0, lm = 0;
                for (int i = 1; i < 19; ++i) {
                    const int xn = (x + CX[i] + nx) % nx, yn = (y + CY[i] + ny) % ny,
                              zn = (z + CZ[i] + nz) % nz;
                    const uint8_t cn = s->flags[(uint64_t(zn) * ny + yn) * nx + xn];
                    if (cn == STRO_FLUID) continue;
                    sm |= 1u << (i - 1);
                    if (cn == STRO_LID || cn == STRO_INFLOW || cn == STRO_OUTFLOW) lm |= 1u << (i - 1);
                }
                s->smask[idx] = sm;
                s->lmask[idx] = lm;
            }
    if (!geo_on(s) && !s->force_geometry) return STRO_OK;
    std::vector<uint8_t> cell(N);
    std::vector<uint32_t> geo(N);
    for (uint64_t n = 0; n < N; ++n) {
        const uint8_t c = s->flags[n];
        const bool e = s->has_eps && s->eps[n] != 0.0f && c == STRO_FLUID;
        cell[n] = uint8_t((c & CELL_TYPE_MASK) | (e ? CELL_EPS_BIT : 0));
        uint32_t g = s->smask[n];
        if (e) g |= GEO_EPS;
        if (s->lmask[n]) g |= GEO_MOVING;
        if (c != STRO_FLUID) g |= GEO_NONFLUID;
        geo[n] = g;
    }
    if (!s->d_cell) {
        STRO_CUDA(cudaMalloc(&s->d_cell, N));
        STRO_CUDA(cudaMalloc(&s->d_geo, N * 4));
        STRO_CUDA(cudaMalloc(&s->d_lmask, N * 4));
    }
    cudaStream_t st = s->ctx->stream;
    STRO_CUDA(cudaMemcpyAsync(s->d_cell, cell.data(), N, cudaMemcpyHostToDevice, st));
    STRO_CUDA(cudaMemcpyAsync(s->d_geo, geo.data(), N * 4, cudaMemcpyHostToDevice, st));
    STRO_CUDA(cudaMemcpyAsync(s->d_lmask, s->lmask.data(), N * 4, cudaMemcpyHostToDevice, st));
    STRO_CUDA(cudaStreamSynchronize(st));
    s->cell_host.swap(cell);
    s->geo_host.swap(geo);
    ++s->geo_version;
    return STRO_OK;
}

void free_sim(stro_sim* s) {
    drop_graphs(s);
    cudaFree(s->d_f);
    cudaFree(s->d_cell);
    cudaFree(s->d_geo);
    cudaFree(s->d_lmask);
    cudaFree(s->d_eps);
    cudaFree(s->d_render);
    cudaFree(s->d_ffield);
    cudaFree(s->d_moments);
    cudaFree(s->d_partials);
    cudaFree(s->d_out);
    cudaFree(s->d_error);
    cudaFree(s->d_blocks);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
}

int launch_one_step(stro_sim* s, int64_t t, bool probe, const int box[4]) {
    StepArgs a = step_args(s, t);
    if (probe) {
        a.box_x0 = box[0]; a.box_x1 = box[1]; a.box_y0 = box[2]; a.box_y1 = box[3];
    }
    const cudaError_t e = launch_sim_step(s, a, t, probe);
    if (e != cudaSuccess) return cuda_fail(e, "step launch");
    return STRO_OK;
}

int run_steps(stro_sim* s, int64_t steps, int64_t probe_step = -1, const int* box = nullptr) {
    cudaStream_t st = s->ctx->stream;
    STRO_CUDA(cudaEventRecord(s->ev0, st));
    const int64_t t0 = s->steps_done, t1 = t0 + steps;
    const int64_t G = steps >= 2 * kRunGraphSteps ? kRunGraphSteps : 0;
    int rc;
    if (probe_step >= t0 && probe_step < t1) {
        rc = launch_plain_steps(s, t0, probe_step - t0, G);
        if (rc == STRO_OK) rc = launch_one_step(s, probe_step, true, box);
        if (rc == STRO_OK) rc = launch_plain_steps(s, probe_step + 1, t1 - probe_step - 1, G);
    } else {
        rc = launch_plain_steps(s, t0, steps, G);
    }
    if (rc != STRO_OK) return rc;
    STRO_CUDA(cudaEventRecord(s->ev1, st));
    STRO_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0.0f;
    STRO_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->gpu_seconds += double(ms) * 1e-3;
    s->steps_done += steps;
    STRO_CUDA(cudaGetLastError());
    return check_rows_error(s);
}

// The row-staged variant records a bulk-copy wait that gave up in a device
// word (the kernel returns instead of waiting on): read it after a run, reset
// it and report the timeout.
int check_rows_error(stro_sim* s) {
    if (s->variant != 2) return STRO_OK;
    int err = 0;
    cudaStream_t st = sim_stream(s);
    STRO_CUDA(cudaMemcpyAsync(&err, s->d_error, sizeof err, cudaMemcpyDeviceToHost, st));
    STRO_CUDA(cudaStreamSynchronize(st));
    if (err == 0) return STRO_OK;
    cudaMemsetAsync(s->d_error, 0, sizeof(int), st);  // ordered before the next launch
    return fail(STRO_ERR_TIMEOUT, "a bulk-copy wait of the row-staged step timed out");
}

int ensure_partials(stro_sim* s, size_t doubles) {
    if (s->partials_len >= doubles) return STRO_OK;
    cudaFree(s->d_partials);
    s->d_partials = nullptr;
    STRO_CUDA(cudaMalloc(&s->d_partials, doubles * sizeof(double)));
    s->partials_len = doubles;
    return STRO_OK;
}

// Bulk / boundary block lists for the current block shape (rebuilt when the
// shape or the geometry changes). A block is bulk when every cell it covers is
// fluid with no wall neighbour, no moving wall nearby and no solid fraction.
// Whether cell (x, y, z) is one the x-face kernels (odd_cell_xface) compute
// as the wall-aware ones do: a velocity-inflow cell of column 0 or nx - 1, or a
// fluid cell without solid fraction whose wall links are exactly its links
// into those columns, all of them into inflow cells.
static bool xface_cell(const stro_sim* s, int x, int y, int z) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const uint64_t idx = (uint64_t(z) * ny + y) * nx + x;
    if (x == 0 || x == nx - 1) return s->flags[idx] == STRO_INFLOW;
    if (s->flags[idx] != STRO_FLUID || s->cell_host[idx] != 0) return false;
    uint32_t expect = 0;
    for (int i = 1; i < 19; ++i)
        if ((x == 1 && CX[i] < 0) || (x == nx - 2 && CX[i] > 0)) expect |= 1u << (i - 1);
    if (s->smask[idx] != expect || s->lmask[idx] != expect) return false;
    for (int i = 1; i < 19; ++i) {
        if (!((expect >> (i - 1)) & 1u)) continue;
        const int xn = x + CX[i], yn = (y + CY[i] + ny) % ny, zn = (z + CZ[i] + nz) % nz;
        if (s->flags[(uint64_t(zn) * ny + yn) * nx + xn] != STRO_INFLOW) return false;
    }
    return true;
}

void block_lists(const stro_sim* s, dim3 shape, std::vector<uint32_t>& bulk,
                 std::vector<uint32_t>& edge, std::vector<uint32_t>* face) {
    const uint32_t bx = shape.x, by = shape.y;
    const uint32_t gx = (uint32_t(s->nx) + bx - 1) / bx, gy = (uint32_t(s->ny) + by - 1) / by;
    const uint64_t nblocks = uint64_t(gx) * gy * uint64_t(s->nz);
    bulk.clear();
    edge.clear();
    if (face) face->clear();
    bulk.reserve(nblocks);
    for (uint64_t b = 0; b < nblocks; ++b) {
        const uint32_t bxi = uint32_t(b % gx), t = uint32_t(b / gx), byi = t % gy, z = t / gy;
        const uint32_t y1 = std::min<uint32_t>((byi + 1) * by, s->ny);
        const uint32_t x1 = std::min<uint32_t>((bxi + 1) * bx, s->nx);
        bool is_bulk = true;
        for (uint32_t yy = byi * by; yy < y1 && is_bulk; ++yy) {
            const uint64_t row = (uint64_t(z) * s->ny + yy) * s->nx;
            for (uint32_t xx = bxi * bx; xx < x1; ++xx)
                if (s->cell_host[row + xx] != 0 || s->geo_host[row + xx] != 0) {
                    is_bulk = false;
                    break;
                }
        }
        if (is_bulk) {
            bulk.push_back(uint32_t(b));
            continue;
        }
        bool is_face = face != nullptr;
        for (uint32_t yy = byi * by; yy < y1 && is_face; ++yy)
            for (uint32_t xx = bxi * bx; xx < x1 && is_face; ++xx)
                is_face = xface_cell(s, int(xx), int(yy), int(z));
        (is_face ? *face : edge).push_back(uint32_t(b));
    }
}

// Feature level of wall-free cells (no solid fraction among them).
static int bulk_feat(const stro_sim* s) {
    if (s->collision == STRO_COLLISION_KBC) return 3;
    if (s->c_smago > 0.0f) return 2;
    return (sponge_active(s) || force_on(s)) ? 1 : 0;
}

// Split modes 4 and 5: bulk and x-face blocks run in one launch, from one
// merged list; mode 5 takes FP16 bulk blocks two cells per thread where the
// pair kernels apply.
static bool merged_split(const stro_sim* s) {
    return (s->merged_faces || s->pair_bulk) && s->face_lists;
}
static bool pair_split(const stro_sim* s) {
    return s->pair_bulk && merged_split(s) &&
           exact::kPair.list_supported(s->precision == STRO_FP16S ? 1 : 0, bulk_feat(s), s->nx,
                                       s->plane, s->block);
}

// d_blocks holds the bulk, x-face and edge lists one after another; in split
// modes 4 and 5 the bulk and x-face blocks form one list in block order (x-face
// entries flagged kListFaceBit), so a bulk block and the x-face block beside it
// run at about the same time and share the DRAM lines they both touch.
static int ensure_block_lists(stro_sim* s) {
    const bool merged = merged_split(s);
    if (s->lists_version == s->geo_version && s->lists_block.x == s->block.x &&
        s->lists_block.y == s->block.y && s->lists_face == s->face_lists &&
        s->lists_merged == merged)
        return STRO_OK;
    const uint32_t bx = s->block.x, by = s->block.y;
    const uint32_t gx = (uint32_t(s->nx) + bx - 1) / bx, gy = (uint32_t(s->ny) + by - 1) / by;
    const uint64_t nblocks = uint64_t(gx) * gy * uint64_t(s->nz);
    std::vector<uint32_t> bulk, edge, face;
    block_lists(s, s->block, bulk, edge, s->face_lists ? &face : nullptr);
    // Launches of this lattice still in flight read the old lists: let them
    // finish before the buffer is released. The new lists go up on the
    // lattice's own stream, so every launch after this call is ordered behind
    // the copy. (A plain cudaMemcpy runs on the legacy default stream, which
    // this non-blocking stream does not wait for, and from pageable memory it
    // may return before its DMA has landed: a launch could then read a fresh,
    // uninitialised allocation.)
    cudaStream_t st = sim_stream(s);
    STRO_CUDA(cudaStreamSynchronize(st));
    cudaFree(s->d_blocks);
    s->d_blocks = nullptr;
    STRO_CUDA(cudaMalloc(&s->d_blocks, std::max<size_t>(nblocks, 1) * sizeof(uint32_t)));
    s->nbulk = uint32_t(bulk.size());
    s->nface = uint32_t(face.size());
    s->nedge = uint32_t(edge.size());
    std::vector<uint32_t> all;
    all.reserve(nblocks);
    if (merged) {
        size_t i = 0, j = 0;  // both lists ascend in block index
        while (i < bulk.size() || j < face.size()) {
            if (j == face.size() || (i < bulk.size() && bulk[i] < face[j])) all.push_back(bulk[i++]);
            else all.push_back(face[j++] | kListFaceBit);
        }
    } else {
        all = bulk;
        all.insert(all.end(), face.begin(), face.end());
    }
    all.insert(all.end(), edge.begin(), edge.end());
    STRO_CUDA(cudaMemcpyAsync(s->d_blocks, all.data(), nblocks * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, st));
    STRO_CUDA(cudaStreamSynchronize(st));  // `all` is released on return
    s->lists_block = s->block;
    s->lists_version = s->geo_version;
    s->lists_face = s->face_lists;
    s->lists_merged = merged;
    return STRO_OK;
}

cudaError_t launch_sim_step(stro_sim* s, const StepArgs& a, int64_t t, bool probe) {
    const int half = s->precision == STRO_FP16S ? 1 : 0;
    const int geo = geo_on(s) ? 1 : 0;
    const bool fused = s->arith == STRO_ARITH_FUSED;
    const StepLaunchers& L = fused ? fused::kStep : exact::kStep;
    const RowsLaunchers& R = fused ? fused::kRows : exact::kRows;
    if (geo && !probe && s->variant == 0 && s->split && s->geo_host.size() == s->N) {
        if (ensure_block_lists(s) != STRO_OK) return cudaErrorMemoryAllocation;
        const bool merged = s->lists_merged, pair = merged && pair_split(s);
        s->last_path = pair ? "split-pair" : (merged ? "split-merged" : "split");
        if (pair) {
            const PairLaunchers& PL = fused ? fused::kPair : exact::kPair;
            const cudaError_t e = PL.list_launch(a, int(t & 1), bulk_feat(s), s->block,
                                                 s->d_blocks, s->nbulk + s->nface, sim_stream(s));
            if (e != cudaSuccess) return e;
        }
        return L.split(a, half, int(t & 1), bulk_feat(s), feat_on(s), s->block, s->d_blocks,
                       pair ? 0u : (merged ? s->nbulk + s->nface : s->nbulk),
                       s->d_blocks + s->nbulk, merged ? 0u : s->nface,
                       s->d_blocks + s->nbulk + s->nface, s->nedge, s->edge_colmajor ? 1 : 0,
                       merged ? 1 : 0, sim_stream(s));
    }
    const PairLaunchers& PL = fused ? fused::kPair : exact::kPair;
    const bool kbc = s->collision == STRO_COLLISION_KBC;  // one-cell kernels only
    if (!kbc && s->variant == 1 && PL.supported(half, geo, probe, s->nx, s->plane, s->pair_block)) {
        s->last_path = "pair";
        return PL.launch(a, int(t & 1), feat_on(s), s->pair_block, sim_stream(s));
    }
    if (!kbc && (s->variant == 4 || s->variant == 5)) {
        const int cells = s->variant == 4 ? 4 : 8;
        if (PL.wide_supported(half, geo, probe, s->nx, s->ny, s->plane, s->block, cells)) {
            s->last_path = cells == 4 ? "wide4" : "wide8";
            return PL.wide_launch(a, int(t & 1), feat_on(s), s->block, cells, sim_stream(s));
        }
    }
    if (!kbc && s->variant == 3 && !geo && !probe && s->block.x * s->block.y <= 128) {
        s->last_path = "capped";
        return L.capped(a, half, int(t & 1), feat_on(s), s->block, sim_stream(s));
    }
    if (!kbc && s->variant == 2 &&
        R.supported(half, geo, probe, s->nx, s->ny, s->rows_threads, s->rows_per_tile)) {
        s->last_path = "rows";
        return R.launch(a, half, int(t & 1), feat_on(s), s->rows_threads, s->rows_per_tile,
                        s->ctx->sm_count, s->d_error, s->rows_polls, sim_stream(s));
    }
    s->last_path = probe ? "probe" : "cell";
    return L.step(a, half, int(t & 1), geo, feat_on(s), probe, probe ? s->probe_block : s->block,
                  sim_stream(s));
}

// ---- CUDA graphs of plain steps ---------------------------------------------
// Once the inflow / lid ramp is over, a step's launches depend only on its
// parity, so a run of G plain steps (G even) is the same launch sequence each
// time. It is captured once and replayed with one cudaGraphLaunch: on lattices
// of a few hundred thousand cells the host's per-kernel launch cost and the gaps
// between dependent launches are a large part of a step.

void drop_graphs(stro_sim* s) {
    for (auto& g : s->graph_cache) cudaGraphExecDestroy(g.second);
    s->graph_cache.clear();
}

namespace {

constexpr size_t kGraphCacheSize = 4;

template <typename T>
void put_bytes(std::vector<uint8_t>& k, const T& v) {
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
    k.insert(k.end(), p, p + sizeof(T));
}

// Everything the launches of a plain step at parity (t & 1) read from the
// simulation: its arguments (ramp over, so the same for every t of that
// parity) and the launch configuration.
std::vector<uint8_t> graph_key(const stro_sim* s, int64_t t, int64_t G) {
    std::vector<uint8_t> k;
    StepArgs a;
    std::memset(&a, 0, sizeof a);
    fill_step_args(s, t, &a);
    put_bytes(k, a);
    const int64_t cfg[] = {t & 1, G, s->variant, s->split ? 1 : 0, s->edge_colmajor ? 1 : 0,
                           s->block.x, s->block.y,
                           s->pair_block.x, s->pair_block.y, s->rows_threads, s->rows_per_tile,
                           s->arith, s->collision, s->precision, geo_on(s) ? 1 : 0, feat_on(s),
                           bulk_feat(s), int64_t(reinterpret_cast<uintptr_t>(s->d_blocks)),
                           s->nbulk, s->nface, s->nedge, int64_t(s->lists_version),
                           s->face_lists ? 1 : 0, s->lists_face ? 1 : 0, s->pair_bulk ? 1 : 0,
                           s->merged_faces ? 1 : 0, s->lists_merged ? 1 : 0,
                           int64_t(s->geo_version), s->lists_block.x, s->lists_block.y,
                           int64_t(reinterpret_cast<uintptr_t>(s->d_error)), s->rows_polls,
                           s->ctx->sm_count,
                           int64_t(reinterpret_cast<uintptr_t>(sim_stream(s)))};
    put_bytes(k, cfg);
    return k;
}

}  // namespace

// Capture G steps starting at parity (t & 1). The block lists of the split are
// built before the capture, so nothing inside it allocates or copies
// synchronously. (The row-staged variant sets kernel attributes at its first
// launch and is not captured.)
static int graph_for(stro_sim* s, int64_t t, int64_t G, cudaGraphExec_t* out) {
    if (geo_on(s) && s->variant == 0 && s->split && s->geo_host.size() == s->N) {
        const int rc = ensure_block_lists(s);
        if (rc != STRO_OK) return rc;
    }
    std::vector<uint8_t> key = graph_key(s, t, G);
    for (size_t i = 0; i < s->graph_cache.size(); ++i)
        if (s->graph_cache[i].first == key) {
            *out = s->graph_cache[i].second;
            return STRO_OK;
        }
    cudaStream_t st = sim_stream(s);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "step graph capture");
    cudaError_t le = cudaSuccess;
    for (int64_t j = 0; j < G && le == cudaSuccess; ++j)
        le = launch_sim_step(s, step_args(s, t + j), t + j, false);
    e = cudaStreamEndCapture(st, &graph);
    if (le != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(le, "step launch (graph capture)");
    }
    if (e != cudaSuccess) return cuda_fail(e, "step graph capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "step graph instantiate");
    if (s->graph_cache.size() >= kGraphCacheSize) {
        cudaGraphExecDestroy(s->graph_cache.front().second);
        s->graph_cache.erase(s->graph_cache.begin());
    }
    s->graph_cache.emplace_back(std::move(key), exec);
    *out = exec;
    return STRO_OK;
}

int launch_plain_steps(stro_sim* s, int64_t t, int64_t count, int64_t graph_steps) {
    const int64_t end = t + count;
    const bool graphs = s->graphs && s->variant != 2 && graph_steps >= 2 && graph_steps % 2 == 0;
    // ramped steps go one by one (their arguments change every step)
    const int64_t ramp_end = s->ramp_steps > 0 ? std::max<int64_t>(t, s->ramp_steps) : t;
    int64_t k = t;
    for (; k < end && (k < ramp_end || !graphs); ++k) {
        const int rc = launch_one_step(s, k, false, nullptr);
        if (rc != STRO_OK) return rc;
    }
    if (graphs && end - k >= graph_steps) {
        cudaGraphExec_t exec = nullptr;
        const int rc = graph_for(s, k, graph_steps, &exec);
        if (rc != STRO_OK) return rc;
        for (; end - k >= graph_steps; k += graph_steps)
            STRO_CUDA(cudaGraphLaunch(exec, sim_stream(s)));
    }
    for (; k < end; ++k) {
        const int rc = launch_one_step(s, k, false, nullptr);
        if (rc != STRO_OK) return rc;
    }
    return STRO_OK;
}

void ctx_retain(stro_ctx* c) { ++c->refs; }

void ctx_release(stro_ctx* c) {
    if (--c->refs > 0) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int ensure_geometry(stro_sim* s) {
    if (s->d_cell) return STRO_OK;
    s->force_geometry = true;
    return upload_geometry(s);
}

int sampled_begin(stro_sim* s, int64_t transient, int64_t sample_steps, int64_t stride,
                  const int32_t box_in[4], double* forces, int64_t capacity, int64_t* samples,
                  int64_t* steps_at, SampledRun* run) {
    const int32_t x0 = box_in[0], x1 = box_in[1], y0 = box_in[2], y1 = box_in[3];
    if (!samples) return fail(STRO_ERR_INVALID, "null sample count");
    if (!s->wants_forces) return fail(STRO_ERR_STATE, "force samples require wants_forces");
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "a sampled run must start at an even step count");
    if (transient < 0 || sample_steps < 0 || stride < 1)
        return fail(STRO_ERR_INVALID, "negative step counts or stride < 1");
    if (x0 < 0 || x1 >= s->nx || y0 < 0 || y1 >= s->ny || x0 > x1 || y0 > y1)
        return fail(STRO_ERR_INVALID, "force box outside the lattice");
    // Ladder.measure (Ladder.swift:55-66): even transient, then chunks of
    // max(2, stride - 2) rounded down to even steps, each followed by the
    // two-step force probe, until sample_steps steps are taken
    transient &= ~int64_t(1);
    const int64_t chunk = std::max<int64_t>(2, stride - 2) & ~int64_t(1);
    const int64_t n = (sample_steps + chunk + 1) / (chunk + 2);
    *samples = n;
    if (n > capacity || (n > 0 && !forces)) {
        return fail(STRO_ERR_INVALID, "sample buffer holds " + std::to_string(capacity) +
                                          " samples, the run takes " + std::to_string(n));
    }
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = sim_stream(s);
    *run = SampledRun{};
    if (n > 0) STRO_CUDA(cudaMalloc(&run->d_samples, size_t(n) * 3 * sizeof(double)));
    cudaError_t e = cudaSuccess;
    if (n > 0) e = cudaMemsetAsync(run->d_samples, 0, size_t(n) * 3 * sizeof(double), st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev0, st);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(st);
        cudaFree(run->d_samples);
        run->d_samples = nullptr;
        return cuda_fail(e, "sampled run");
    }
    run->forces = forces;
    run->count = n;
    run->steps_at = steps_at;
    run->t = s->steps_done;
    run->transient_left = transient;
    run->chunk = chunk;
    std::copy(box_in, box_in + 4, run->box);
    // plain steps replay CUDA graphs: one of `chunk` steps per sample when it
    // is short, else runs of 32
    run->g_transient = transient >= 2 * kRunGraphSteps ? kRunGraphSteps : 0;
    run->g_chunk = (n >= 2 && chunk <= 256) ? chunk
                                            : (chunk >= 2 * kRunGraphSteps ? kRunGraphSteps : 0);
    return STRO_OK;
}

int sampled_advance(stro_sim* s, SampledRun* run) {
    if (run->done) return STRO_OK;
    cudaStream_t st = sim_stream(s);
    if (run->transient_left > 0) {  // the transient, in pieces of 1024 steps
        const int64_t piece = std::min<int64_t>(run->transient_left, 1024);
        const int rc = launch_plain_steps(s, run->t, piece, run->g_transient);
        run->t += piece;
        run->transient_left -= piece;
        return rc;
    }
    if (run->k < run->count) {  // one sample: the chunk, then the probe pair
        int rc = launch_plain_steps(s, run->t, run->chunk, run->g_chunk);
        run->t += run->chunk;
        const bool geo = geo_on(s);
        for (int j = 0; j < 2 && rc == STRO_OK; ++j, ++run->t)  // the force is taken on the odd step
            rc = launch_one_step(s, run->t, geo && j == 1, run->box);
        if (rc != STRO_OK) return rc;
        if (geo) {
            const dim3 pgrid = step_grid(step_args(s, 0), s->probe_block);
            const int nblocks = int(pgrid.x * pgrid.y * pgrid.z);
            STRO_CUDA(launch_fold(s->d_partials, nblocks, 3, run->d_samples + 3 * run->k, st));
        }
        if (run->steps_at) run->steps_at[run->k] = run->t;
        ++run->k;
        return STRO_OK;
    }
    cudaError_t e = cudaEventRecord(s->ev1, st);
    if (e == cudaSuccess && run->count > 0)
        e = cudaMemcpyAsync(run->forces, run->d_samples, size_t(run->count) * 3 * sizeof(double),
                            cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(e, "sampled run");
    run->done = true;
    return STRO_OK;
}

int sampled_finish(stro_sim* s, SampledRun* run) {
    cudaSetDevice(s->ctx->device);
    const cudaError_t e = cudaStreamSynchronize(sim_stream(s));
    cudaFree(run->d_samples);
    run->d_samples = nullptr;
    if (e != cudaSuccess) return cuda_fail(e, "sampled run");
    if (!run->done) return STRO_OK;  // abandoned after an error: only freed
    float ms = 0.0f;
    STRO_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->gpu_seconds += double(ms) * 1e-3;
    s->steps_done = run->t;
    return check_rows_error(s);
}

}  // namespace rt
}  // namespace stro

int stro::rt::observables(stro_sim* s, double out[2]) {
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "observables require an even step count");
    cudaSetDevice(s->ctx->device);
    STRO_CUDA(launch_observables(field_view(s), s->precision == STRO_FP16S, s->omega,
                                 s->d_partials, s->d_out, s->ctx->stream));
    STRO_CUDA(cudaMemcpyAsync(out, s->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return STRO_OK;
}

#define CHECK_SIM(s) \
    if (!(s)) return fail(STRO_ERR_INVALID, "null simulation handle")

extern "C" {

const char* stro_last_error(void) { return g_error.c_str(); }
int stro_abi_version(void) { return STRO_ABI_VERSION; }

int stro_ctx_create(int device, stro_ctx** out) {
    if (!out) return fail(STRO_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(STRO_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= count) return fail(STRO_ERR_INVALID, "device index out of range");
    STRO_CUDA(cudaSetDevice(device));
    stro_ctx* c = new (std::nothrow) stro_ctx;
    if (!c) return fail(STRO_ERR_OOM, "host allocation failed");
    c->device = device;
    cudaDeviceProp prop{};
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "context set-up");
    }
    c->sm_count = prop.multiProcessorCount;
    std::snprintf(c->name, sizeof c->name, "%s", prop.name);
    *out = c;
    return STRO_OK;
}

int stro_ctx_destroy(stro_ctx* ctx) {
    if (!ctx || ctx->closed) return STRO_OK;
    ctx->closed = true;
    ctx_release(ctx);
    return STRO_OK;
}

int stro_ctx_info(stro_ctx* ctx, char* name, size_t name_len, int* sm_count) {
    if (!ctx) return fail(STRO_ERR_INVALID, "null context");
    if (name && name_len) std::snprintf(name, name_len, "%s", ctx->name);
    if (sm_count) *sm_count = ctx->sm_count;
    return STRO_OK;
}

int stro_sim_create(stro_ctx* ctx, const stro_sim_desc* d, const uint8_t* flags, stro_sim** out) {
    if (!ctx || !d || !out) return fail(STRO_ERR_INVALID, "null argument");
    *out = nullptr;
    if (ctx->closed) return fail(STRO_ERR_INVALID, "context already destroyed");
    if (d->precision != STRO_FP32 && d->precision != STRO_FP16S)
        return fail(STRO_ERR_INVALID, "precision must be STRO_FP32 or STRO_FP16S");
    if (d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nx > 65535 * 256 || d->ny > 65535 ||
        d->nz > 65535)
        return fail(STRO_ERR_INVALID, "lattice dimensions out of range");
    const uint64_t N = uint64_t(d->nx) * d->ny * d->nz;
    if (N >= (1ull << 31) || 19ull * (N + 64) >= (1ull << 40))
        return fail(STRO_ERR_INVALID, "lattice too large (N must be < 2^31 cells)");
    if (flags)
        for (uint64_t n = 0; n < N; ++n)
            if (flags[n] > STRO_OUTFLOW) return fail(STRO_ERR_INVALID, "flag value out of range");
    STRO_CUDA(cudaSetDevice(ctx->device));
    stro_sim* s = new (std::nothrow) stro_sim;
    if (!s) return fail(STRO_ERR_OOM, "host allocation failed");
    s->ctx = ctx;
    s->precision = d->precision;
    s->nx = d->nx; s->ny = d->ny; s->nz = d->nz;
    s->N = N;
    s->plane = padded_plane(N);
    s->esize = d->precision == STRO_FP16S ? 2 : 4;
    s->omega = d->omega;
    s->omega_minus = d->omega_minus;
    std::memcpy(s->lid, d->lid, sizeof s->lid);
    s->uin = d->uin;
    s->ramp_steps = d->ramp_steps;
    std::memcpy(s->force, d->force, sizeof s->force);
    s->c_smago = d->c_smago;
    s->wants_forces = d->wants_forces != 0;
    s->block = default_block(d->nx);
    s->probe_block = s->block;
    if (d->precision == STRO_FP16S && d->nx % 64 == 0) {
        // FP16 lattices with whole warps of cell pairs per row default to the pair variant
        int bxp = std::min(256, d->nx / 2);
        while ((d->nx / 2) % bxp != 0) bxp -= 32;
        s->pair_block = dim3(bxp, 1, 1);
        s->variant = 1;
    }
    try {
        s->flags.assign(N, 0);
        if (flags) std::memcpy(s->flags.data(), flags, N);
    } catch (const std::bad_alloc&) {
        delete s;
        return fail(STRO_ERR_OOM, "host allocation failed");
    }
    auto bail = [&](int rc) {
        free_sim(s);
        delete s;
        return rc;
    };
    cudaError_t e = cudaMalloc(&s->d_f, 19 * s->plane * s->esize);
    if (e != cudaSuccess) return bail(cuda_fail(e, "DDF allocation"));
    // shifted equilibrium at rest is exactly 0 (Sim.swift:225)
    e = cudaMemsetAsync(s->d_f, 0, 19 * s->plane * s->esize, ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_out, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_error, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_error, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess) return bail(cuda_fail(e, "simulation set-up"));
    int rc = upload_geometry(s);
    if (rc != STRO_OK) return bail(rc);
    const dim3 grid = dim3((s->nx + s->probe_block.x - 1) / s->probe_block.x,
                           (s->ny + s->probe_block.y - 1) / s->probe_block.y, s->nz);
    const size_t step_blocks = size_t(grid.x) * grid.y * grid.z;
    rc = ensure_partials(s, std::max<size_t>(s->wants_forces ? 3 * step_blocks : 0, 2 * 2048));
    if (rc != STRO_OK) return bail(rc);
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "simulation set-up"));
    ctx_retain(ctx);
    *out = s;
    return STRO_OK;
}

int stro_sim_destroy(stro_sim* s) {
    if (!s) return STRO_OK;
    stro_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_sim(s);
    delete s;
    ctx_release(c);
    return STRO_OK;
}

int stro_sim_set_omega(stro_sim* s, float omega, float omega_minus) {
    CHECK_SIM(s);
    s->omega = omega;
    s->omega_minus = omega_minus;
    return STRO_OK;
}
int stro_sim_set_lid(stro_sim* s, const float lid[3]) {
    CHECK_SIM(s);
    if (!lid) return fail(STRO_ERR_INVALID, "null lid");
    std::memcpy(s->lid, lid, sizeof s->lid);
    return STRO_OK;
}
int stro_sim_set_uin(stro_sim* s, float uin) {
    CHECK_SIM(s);
    s->uin = uin;
    return STRO_OK;
}
int stro_sim_set_ramp_steps(stro_sim* s, int32_t r) {
    CHECK_SIM(s);
    s->ramp_steps = r;
    return STRO_OK;
}
int stro_sim_set_force(stro_sim* s, const float f[3]) {
    CHECK_SIM(s);
    if (!f) return fail(STRO_ERR_INVALID, "null force");
    std::memcpy(s->force, f, sizeof s->force);
    return STRO_OK;
}
int stro_sim_set_c_smago(stro_sim* s, float c) {
    CHECK_SIM(s);
    if (c > 0.0f && s->collision == STRO_COLLISION_KBC)
        return fail(STRO_ERR_INVALID, "the KBC collision has no Smagorinsky model");
    s->c_smago = c;
    return STRO_OK;
}
int stro_sim_set_inflow_uniform(stro_sim* s, int u) {
    CHECK_SIM(s);
    s->inflow_uniform = u ? 1 : 0;
    return STRO_OK;
}
int stro_sim_set_sponge(stro_sim* s, int enabled, float x0, float width, float tau) {
    CHECK_SIM(s);
    if (enabled && !(width > 0.0f)) return fail(STRO_ERR_INVALID, "sponge width must be > 0");
    s->sponge_on = enabled != 0;
    s->sponge_x0 = enabled ? x0 : 1e9f;
    s->sponge_width = enabled ? width : 0.0f;
    s->sponge_tau = enabled ? tau : 1.0f;
    return STRO_OK;
}

int stro_sim_set_solid_fractions(stro_sim* s, const float* eps) {
    CHECK_SIM(s);
    if (!eps) return fail(STRO_ERR_INVALID, "null eps");
    if (s->collision == STRO_COLLISION_KBC)
        for (uint64_t n = 0; n < s->N; ++n)
            if (eps[n] > 0.0f)
                return fail(STRO_ERR_INVALID, "the KBC collision has no partially solid cells");
    cudaSetDevice(s->ctx->device);
    s->eps.assign(eps, eps + s->N);
    s->has_eps = true;
    if (!s->d_eps) STRO_CUDA(cudaMalloc(&s->d_eps, s->N * 4));
    STRO_CUDA(cudaMemcpyAsync(s->d_eps, eps, s->N * 4, cudaMemcpyHostToDevice, s->ctx->stream));
    return upload_geometry(s);
}

int stro_sim_set_force_field(stro_sim* s, const float* fxyz) {
    CHECK_SIM(s);
    cudaSetDevice(s->ctx->device);
    if (!fxyz) {
        s->has_ffield = false;
        return STRO_OK;
    }
    if (!s->d_ffield) STRO_CUDA(cudaMalloc(&s->d_ffield, 3 * s->N * 4));
    STRO_CUDA(cudaMemcpyAsync(s->d_ffield, fxyz, 3 * s->N * 4, cudaMemcpyHostToDevice,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    s->has_ffield = true;
    // An all-zero field adds exact zeros to the uniform force: the step skips the
    // field (and, with no uniform force, the Guo terms), with identical results.
    s->ffield_nonzero = false;
    for (uint64_t k = 0; k < 3 * s->N && !s->ffield_nonzero; ++k) s->ffield_nonzero = fxyz[k] != 0.0f;
    return STRO_OK;
}

int stro_sim_init_field(stro_sim* s, uint32_t mode, float amplitude) {
    CHECK_SIM(s);
    if (mode > 2) return fail(STRO_ERR_INVALID, "init mode must be 0, 1 or 2");
    cudaSetDevice(s->ctx->device);
    const float tau = 1.0f / s->omega;
    STRO_CUDA(launch_init_field(field_view(s), s->precision == STRO_FP16S, mode, amplitude, tau,
                                s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return STRO_OK;
}

int stro_sim_state_bytes(stro_sim* s, size_t* bytes) {
    CHECK_SIM(s);
    if (!bytes) return fail(STRO_ERR_INVALID, "null output");
    *bytes = 19 * s->N * s->esize;
    return STRO_OK;
}

// The canonical state (19 planes of N values) to or from the padded device
// planes: one copy when the planes are not padded, else one copy per plane.
static int copy_state(stro_sim* s, void* host, bool to_device) {
    const size_t row = s->N * s->esize, pitch = s->plane * s->esize;
    cudaStream_t st = s->ctx->stream;
    const cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    char* h = static_cast<char*>(host);
    char* d = static_cast<char*>(s->d_f);
    if (pitch == row) {
        STRO_CUDA(cudaMemcpyAsync(to_device ? static_cast<void*>(d) : static_cast<void*>(h),
                                  to_device ? static_cast<void*>(h) : static_cast<void*>(d),
                                  19 * row, kind, st));
    } else {
        for (int i = 0; i < 19; ++i) {
            char* hp = h + size_t(i) * row;
            char* dp = d + size_t(i) * pitch;
            STRO_CUDA(cudaMemcpyAsync(to_device ? static_cast<void*>(dp) : static_cast<void*>(hp),
                                      to_device ? static_cast<void*>(hp) : static_cast<void*>(dp),
                                      row, kind, st));
        }
    }
    STRO_CUDA(cudaStreamSynchronize(st));
    return STRO_OK;
}

int stro_sim_upload_state(stro_sim* s, const void* host, size_t bytes) {
    CHECK_SIM(s);
    if (!host || bytes != 19 * s->N * s->esize)
        return fail(STRO_ERR_INVALID, "state size must be 19*N*element_size bytes");
    cudaSetDevice(s->ctx->device);
    return copy_state(s, const_cast<void*>(host), true);
}

int stro_sim_download_state(stro_sim* s, void* host, size_t bytes) {
    CHECK_SIM(s);
    if (!host || bytes != 19 * s->N * s->esize)
        return fail(STRO_ERR_INVALID, "state size must be 19*N*element_size bytes");
    cudaSetDevice(s->ctx->device);
    return copy_state(s, host, false);
}

int stro_sim_run(stro_sim* s, int64_t steps) {
    CHECK_SIM(s);
    if (steps < 0) return fail(STRO_ERR_INVALID, "negative step count");
    if (steps == 0) return STRO_OK;
    cudaSetDevice(s->ctx->device);
    return run_steps(s, steps);
}

int stro_sim_steps_done(stro_sim* s, int64_t* steps) {
    CHECK_SIM(s);
    if (!steps) return fail(STRO_ERR_INVALID, "null output");
    *steps = s->steps_done;
    return STRO_OK;
}

int stro_sim_set_steps_done(stro_sim* s, int64_t steps) {
    CHECK_SIM(s);
    if (steps < 0) return fail(STRO_ERR_INVALID, "negative step count");
    s->steps_done = steps;
    return STRO_OK;
}

int stro_sim_gpu_seconds(stro_sim* s, double* seconds) {
    CHECK_SIM(s);
    if (!seconds) return fail(STRO_ERR_INVALID, "null output");
    *seconds = s->gpu_seconds;
    return STRO_OK;
}

int stro_sim_moments(stro_sim* s, float* out4) {
    CHECK_SIM(s);
    if (!out4) return fail(STRO_ERR_INVALID, "null output");
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "moments probe requires even step count");
    cudaSetDevice(s->ctx->device);
    if (!s->d_moments) STRO_CUDA(cudaMalloc(&s->d_moments, s->N * sizeof(float4)));
    STRO_CUDA(launch_moments(field_view(s), s->precision == STRO_FP16S, s->d_moments,
                             s->ctx->stream));
    STRO_CUDA(cudaMemcpyAsync(out4, s->d_moments, s->N * sizeof(float4), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return STRO_OK;
}

int stro_sim_run_sampled(stro_sim* s, int64_t transient, int64_t sample_steps, int64_t stride,
                         int32_t x0, int32_t x1, int32_t y0, int32_t y1, double* forces,
                         int64_t capacity, int64_t* samples, int64_t* steps_at) {
    CHECK_SIM(s);
    const int32_t box[4] = {x0, x1, y0, y1};
    SampledRun run;
    int rc = sampled_begin(s, transient, sample_steps, stride, box, forces, capacity, samples,
                           steps_at, &run);
    if (rc != STRO_OK) return rc;
    while (rc == STRO_OK && !run.done) rc = sampled_advance(s, &run);
    const int rf = sampled_finish(s, &run);
    return rc != STRO_OK ? rc : rf;
}

int stro_sim_render_slice(stro_sim* s, int32_t z, float uref, uint16_t* rgba, double* seconds) {
    CHECK_SIM(s);
    if (!rgba) return fail(STRO_ERR_INVALID, "null output");
    if (z < 0 || z >= s->nz) return fail(STRO_ERR_INVALID, "slice outside the lattice");
    if (!(uref > 0.0f)) return fail(STRO_ERR_INVALID, "uref must be positive");
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "rendering requires an even step count");
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    const size_t bytes = size_t(s->nx) * size_t(s->ny) * 4 * sizeof(__half);
    if (s->render_bytes < bytes) {
        cudaFree(s->d_render);
        s->d_render = nullptr;
        s->render_bytes = 0;
        STRO_CUDA(cudaMalloc(&s->d_render, bytes));
        s->render_bytes = bytes;
    }
    STRO_CUDA(cudaEventRecord(s->ev0, st));
    STRO_CUDA(launch_render(field_view(s), s->precision == STRO_FP16S, s->d_eps, uint32_t(z), uref,
                            static_cast<__half*>(s->d_render), st));
    STRO_CUDA(cudaEventRecord(s->ev1, st));
    STRO_CUDA(cudaMemcpyAsync(rgba, s->d_render, bytes, cudaMemcpyDeviceToHost, st));
    STRO_CUDA(cudaStreamSynchronize(st));
    if (seconds) {
        float ms = 0.0f;
        STRO_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        *seconds = double(ms) * 1e-3;
    }
    return STRO_OK;
}

int stro_sim_probe_force(stro_sim* s, int32_t x0, int32_t x1, int32_t y0, int32_t y1,
                         double out[3]) {
    CHECK_SIM(s);
    if (!out) return fail(STRO_ERR_INVALID, "null output");
    if (!s->wants_forces) return fail(STRO_ERR_STATE, "force probe requires wants_forces");
    if (s->steps_done % 2 != 0)
        return fail(STRO_ERR_STATE, "force probe requires even step count");
    if (x0 < 0 || x1 >= s->nx || y0 < 0 || y1 >= s->ny || x0 > x1 || y0 > y1)
        return fail(STRO_ERR_INVALID, "force box outside the lattice");
    cudaSetDevice(s->ctx->device);
    if (!geo_on(s)) {  // no wall and no solid fraction: nothing exchanges momentum
        const int rc = run_steps(s, 2);
        out[0] = out[1] = out[2] = 0.0;
        return rc;
    }
    const int box[4] = {x0, x1, y0, y1};
    int rc = run_steps(s, 2, s->steps_done + 1, box);
    if (rc != STRO_OK) return rc;
    StepArgs a = step_args(s, 0);
    const dim3 grid = step_grid(a, s->probe_block);
    const int nblocks = int(grid.x * grid.y * grid.z);
    STRO_CUDA(launch_fold(s->d_partials, nblocks, 3, s->d_out, s->ctx->stream));
    STRO_CUDA(cudaMemcpyAsync(out, s->d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return STRO_OK;
}


int stro_sim_kinetic_energy(stro_sim* s, double* sum_u2) {
    CHECK_SIM(s);
    if (!sum_u2) return fail(STRO_ERR_INVALID, "null output");
    double o[2];
    const int rc = observables(s, o);
    if (rc == STRO_OK) *sum_u2 = o[0];
    return rc;
}

int stro_sim_observables(stro_sim* s, double out[2]) {
    CHECK_SIM(s);
    if (!out) return fail(STRO_ERR_INVALID, "null output");
    return observables(s, out);
}

int stro_sim_dissipation(stro_sim* s, double* sum_eps) {
    CHECK_SIM(s);
    if (!sum_eps) return fail(STRO_ERR_INVALID, "null output");
    double o[2];
    const int rc = observables(s, o);
    if (rc == STRO_OK) *sum_eps = o[1];
    return rc;
}

int stro_sim_digest(stro_sim* s, char hex[65]) {
    CHECK_SIM(s);
    if (!hex) return fail(STRO_ERR_INVALID, "null output");
    cudaSetDevice(s->ctx->device);
    // Stream the planes through a pinned staging buffer in slices.
    const size_t plane_bytes = s->N * s->esize;
    const size_t slice = std::min<size_t>(plane_bytes, size_t(64) << 20);
    void* stage = nullptr;
    STRO_CUDA(cudaMallocHost(&stage, slice));
    Sha256 h;
    for (int i = 0; i < 19; ++i) {
        const char* src = static_cast<const char*>(s->d_f) + size_t(i) * s->plane * s->esize;
        for (size_t off = 0; off < plane_bytes; off += slice) {
            const size_t len = std::min(slice, plane_bytes - off);
            cudaError_t e = cudaMemcpyAsync(stage, src + off, len, cudaMemcpyDeviceToHost,
                                            s->ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
            if (e != cudaSuccess) {
                cudaFreeHost(stage);
                return cuda_fail(e, "digest download");
            }
            h.update(stage, len);
        }
    }
    cudaFreeHost(stage);
    uint8_t dg[32];
    h.finish(dg);
    sha256_hex(dg, hex);
    return STRO_OK;
}

int stro_sim_mass(stro_sim* s, double* total) {
    CHECK_SIM(s);
    if (!total) return fail(STRO_ERR_INVALID, "null output");
    cudaSetDevice(s->ctx->device);
    STRO_CUDA(launch_mass(field_view(s), s->precision == STRO_FP16S, s->d_partials, s->d_out,
                          s->ctx->stream));
    STRO_CUDA(cudaMemcpyAsync(total, s->d_out, sizeof(double), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return STRO_OK;
}

int stro_sim_check_finite(stro_sim* s, int* all_finite) {
    CHECK_SIM(s);
    if (!all_finite) return fail(STRO_ERR_INVALID, "null output");
    cudaSetDevice(s->ctx->device);
    double bad = 0.0;
    STRO_CUDA(launch_nonfinite(field_view(s), s->precision == STRO_FP16S, s->d_partials,
                               s->d_out, s->ctx->stream));
    STRO_CUDA(cudaMemcpyAsync(&bad, s->d_out, sizeof(double), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    STRO_CUDA(cudaStreamSynchronize(s->ctx->stream));
    *all_finite = bad == 0.0 ? 1 : 0;
    return STRO_OK;
}

int stro_sha256_hex(const void* data, size_t len, char hex[65]) {
    if ((!data && len) || !hex) return fail(STRO_ERR_INVALID, "null argument");
    Sha256 h;
    h.update(data, len);
    uint8_t dg[32];
    h.finish(dg);
    sha256_hex(dg, hex);
    return STRO_OK;
}

int stro_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(STRO_ERR_INVALID, "null output");
    *out = nullptr;
    STRO_CUDA(cudaMallocHost(out, bytes));
    return STRO_OK;
}

int stro_host_free(void* ptr) {
    if (ptr) STRO_CUDA(cudaFreeHost(ptr));
    return STRO_OK;
}

// diskSolidFractions, CaseSetups.swift:6-25.
int stro_disk_solid_fractions(int32_t nx, int32_t ny, double cx, double cy, double r, float* out) {
    if (!out || nx < 1 || ny < 1) return fail(STRO_ERR_INVALID, "bad disk arguments");
    std::fill(out, out + size_t(nx) * ny, 0.0f);
    const double r2 = r * r;
    const int sub = 16;
    const int lo = int(cx - r) - 2, hi = int(cx + r) + 2;
    const int loY = int(cy - r) - 2, hiY = int(cy + r) + 2;
    for (int y = std::max(0, loY); y <= std::min(ny - 1, hiY); ++y)
        for (int x = std::max(0, lo); x <= std::min(nx - 1, hi); ++x) {
            int inside = 0;
            for (int sy = 0; sy < sub; ++sy)
                for (int sx = 0; sx < sub; ++sx) {
                    const double px = double(x) - 0.5 + (double(sx) + 0.5) / double(sub);
                    const double py = double(y) - 0.5 + (double(sy) + 0.5) / double(sub);
                    const double dx = px - cx, dy = py - cy;
                    if (dx * dx + dy * dy <= r2) ++inside;
                }
            out[size_t(y) * nx + x] = float(inside) / float(sub * sub);
        }
    return STRO_OK;
}

// sphereSolidFractions, CaseSetups.swift:68-90, with sub^3 samples per cell.
int stro_sphere_solid_fractions(int32_t nx, int32_t ny, int32_t nz, double cx, double cy,
                                double cz, double r, int32_t sub, float* out) {
    if (!out || nx < 1 || ny < 1 || nz < 1 || sub < 1 || sub > 64)
        return fail(STRO_ERR_INVALID, "bad sphere arguments");
    std::fill(out, out + size_t(nx) * ny * nz, 0.0f);
    const double r2 = r * r;
    for (int z = std::max(0, int(cz - r) - 2); z <= std::min(nz - 1, int(cz + r) + 2); ++z)
        for (int y = std::max(0, int(cy - r) - 2); y <= std::min(ny - 1, int(cy + r) + 2); ++y)
            for (int x = std::max(0, int(cx - r) - 2); x <= std::min(nx - 1, int(cx + r) + 2); ++x) {
                int inside = 0;
                for (int sz = 0; sz < sub; ++sz)
                    for (int sy = 0; sy < sub; ++sy)
                        for (int sx = 0; sx < sub; ++sx) {
                            const double px = double(x) - 0.5 + (double(sx) + 0.5) / double(sub);
                            const double py = double(y) - 0.5 + (double(sy) + 0.5) / double(sub);
                            const double pz = double(z) - 0.5 + (double(sz) + 0.5) / double(sub);
                            const double dx = px - cx, dy = py - cy, dz = pz - cz;
                            if (dx * dx + dy * dy + dz * dz <= r2) ++inside;
                        }
                out[(size_t(z) * ny + y) * nx + x] = float(inside) / float(sub * sub * sub);
            }
    return STRO_OK;
}

}  // extern "C"
