// Triangle-mesh voxelization into Noble-Torczynski solid fractions, and the
// binary STL reader and lat-long sphere generator that feed it
// (StlVoxels.swift:1-144).
//
// meshSolidFractions (StlVoxels.swift:52-117) casts 2x2 sub-rays along +x
// through every (y, z) cell, collects the x-crossings of the mesh, pairs them
// into interior spans and adds each span's exact x-coverage of a cell,
// divided by 4, to that cell's fraction. Here:
//   1. the lattice-space transform vertex * scale + offset runs on the GPU
//      (k_transform), so its roundings follow the device arithmetic contract
//      (-fmad=false) instead of the host compiler's contraction choices;
//   2. the host buckets triangles over the (y, z) cells by their bounding box
//      widened by half a cell, as the reference does; a bucket is a superset
//      of the triangles a sub-ray of the cell can hit, so the crossings are
//      exactly the reference's;
//   3. k_columns gives each busy (y, z) column a block and each of its four
//      sub-rays a warp whose lanes split the candidate triangles; the
//      crossings go to a bounded shared list, lane 0 sorts them and applies
//      the reference's tangency merge, and one thread adds the coverage of
//      the four sub-rays in the reference's (sy, sz) order. No two blocks
//      touch a cell, so the result is deterministic and equal to the
//      sequential loop. (A column can have thousands of candidates near the
//      poles of a lat-long mesh; one thread per column left the kernel
//      latency-bound on a few heavy columns.)
// Every FP32 operation keeps the reference's order; the fractions are
// bitwise equal to the oracle's restatement (orc_mesh_solid_fractions).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "runtime_internal.h"

namespace stro {

namespace {

constexpr int kMaxCrossings = 128;  // crossings one sub-ray may collect

__global__ void k_transform(const float* __restrict__ in, float* __restrict__ out, uint32_t count,
                            float scale, float ox, float oy, float oz) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;  // vertex index
    if (k >= count) return;
    out[3 * k + 0] = in[3 * k + 0] * scale + ox;
    out[3 * k + 1] = in[3 * k + 1] * scale + oy;
    out[3 * k + 2] = in[3 * k + 2] * scale + oz;
}

// One block of four warps per busy (y, z) column; warp w casts sub-ray
// (sy, sz) = (w / 2, w % 2). t: lattice-space triangles (9 floats each),
// start/list: CSR buckets of candidate triangles per column, cols: the busy
// columns. The lanes of a warp split the candidates and append their
// crossings to the warp's shared list (the set of crossings does not depend
// on the order, and it is sorted next); lane 0 sorts it and forms the spans;
// then one thread adds the four sub-rays' coverage to the column in the
// reference's (sy, sz) order, so every cell sees the same sequence of
// additions as in the sequential loop.
__global__ void __launch_bounds__(128) k_columns(const float* __restrict__ t,
                                                 const uint32_t* __restrict__ start,
                                                 const uint32_t* __restrict__ list,
                                                 const uint32_t* __restrict__ cols, int nx,
                                                 int ny, float* __restrict__ eps, int* error) {
    __shared__ float xs[4][kMaxCrossings];
    __shared__ float spans[4][kMaxCrossings];  // (x0, x1) pairs
    __shared__ int nxs[4], nspan[4], overflow;
    const int w = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31u);
    const uint32_t col = cols[blockIdx.x];
    const int y = int(col % uint32_t(ny)), z = int(col / uint32_t(ny));
    const uint32_t b0 = start[col], b1 = start[col + 1];
    if (threadIdx.x < 4) nxs[threadIdx.x] = 0;
    if (threadIdx.x == 0) overflow = 0;
    __syncthreads();
    const int sub = 2;
    const int sy = w / sub, sz = w % sub;
    const float ry = float(y) - 0.5f + (float(sy) + 0.5f) / float(sub);
    const float rz = float(z) - 0.5f + (float(sz) + 0.5f) / float(sub);
    for (uint32_t q = b0 + uint32_t(lane); q < b1; q += 32u) {
        const float* tri = t + 9 * size_t(list[q]);
        const float ax = tri[0], ay = tri[1], az = tri[2];
        const float bx = tri[3], by = tri[4], bz = tri[5];
        const float cx = tri[6], cy = tri[7], cz = tri[8];
        const float d1x = by - ay, d1y = bz - az;
        const float d2x = cy - ay, d2y = cz - az;
        const float denom = d1x * d2y - d1y * d2x;
        if (fabsf(denom) < 1e-12f) continue;  // ray-parallel triangle
        const float px = ry - ay, py = rz - az;
        const float u = (px * d2y - py * d2x) / denom;
        const float v = (d1x * py - d1y * px) / denom;
        if (u < 0.0f || v < 0.0f || u + v > 1.0f) continue;
        const int slot = atomicAdd(&nxs[w], 1);
        if (slot < kMaxCrossings) xs[w][slot] = ax + u * (bx - ax) + v * (cx - ax);
        else overflow = 1;
    }
    __syncthreads();
    if (overflow) {
        if (threadIdx.x == 0) atomicExch(error, 1);
        return;
    }
    if (lane == 0) {
        const int count = nxs[w];
        float* x = xs[w];
        for (int i = 1; i < count; ++i) {  // insertion sort, ascending
            const float key = x[i];
            int j = i - 1;
            while (j >= 0 && x[j] > key) {
                x[j + 1] = x[j];
                --j;
            }
            x[j + 1] = key;
        }
        int ns = 0, k = 0;
        while (count >= 2 && k + 1 < count) {
            if (x[k + 1] - x[k] < 1e-5f) {  // grazing hit
                k += 1;
                continue;
            }
            spans[w][2 * ns] = x[k];
            spans[w][2 * ns + 1] = x[k + 1];
            ++ns;
            k += 2;
        }
        nspan[w] = ns;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    float* ecol = eps + size_t(col) * size_t(nx);
    int touched_lo = nx, touched_hi = -1;  // cells this column wrote (the rest stay 0)
    for (int r = 0; r < 4; ++r)
        for (int s = 0; s < nspan[r]; ++s) {
            const float x0 = spans[r][2 * s], x1 = spans[r][2 * s + 1];
            const int c0 = max(0, int(floorf(x0 + 0.5f)));
            const int c1 = min(nx - 1, int(floorf(x1 + 0.5f)));
            touched_lo = min(touched_lo, c0);
            touched_hi = max(touched_hi, c1);
            for (int x = c0; x <= c1; ++x) {
                const float lo = float(x) - 0.5f, hi = float(x) + 0.5f;
                const float cover = fminf(x1, hi) - fmaxf(x0, lo);
                if (cover > 0.0f) ecol[x] += cover / float(sub * sub);
            }
        }
    for (int x = touched_lo; x <= touched_hi; ++x) ecol[x] = fminf(ecol[x], 1.0f);
}

inline uint32_t rd_u32(const uint8_t* p) {
    uint32_t v;
    std::memcpy(&v, p, 4);
    return v;
}

}  // namespace

}  // namespace stro

using namespace stro;
using namespace stro::rt;

extern "C" {

int stro_stl_triangle_count(const uint8_t* data, size_t len, uint32_t* count) {
    if (!data || !count) return fail(STRO_ERR_INVALID, "null argument");
    if (len < 84) return fail(STRO_ERR_INVALID, "STL too short");
    // "solid" at the start and too short for a binary body: ASCII STL
    if (len < 84 + 50) {
        char head[6] = {0};
        for (int k = 0; k < 5; ++k) {
            const unsigned char c = data[k];
            head[k] = char(c >= 'A' && c <= 'Z' ? c - 'A' + 'a' : c);
        }
        if (std::strcmp(head, "solid") == 0)
            return fail(STRO_ERR_INVALID, "ASCII STL not supported (binary only)");
    }
    const uint32_t n = rd_u32(data + 80);
    if (len < 84 + size_t(n) * 50) return fail(STRO_ERR_INVALID, "STL truncated (or ASCII; binary only)");
    *count = n;
    return STRO_OK;
}

int stro_stl_parse(const uint8_t* data, size_t len, float* tris, float bounds[6]) {
    uint32_t n = 0;
    const int rc = stro_stl_triangle_count(data, len, &n);
    if (rc != STRO_OK) return rc;
    if (!tris && n > 0) return fail(STRO_ERR_INVALID, "null triangle buffer");
    float lo[3] = {3.4028235e38f, 3.4028235e38f, 3.4028235e38f};
    float hi[3] = {-3.4028235e38f, -3.4028235e38f, -3.4028235e38f};
    for (uint32_t k = 0; k < n; ++k) {
        const uint8_t* rec = data + 84 + size_t(k) * 50 + 12;  // skip the normal
        for (int j = 0; j < 9; ++j) {
            float v;
            std::memcpy(&v, rec + 4 * j, 4);
            tris[9 * size_t(k) + j] = v;
            lo[j % 3] = std::min(lo[j % 3], v);
            hi[j % 3] = std::max(hi[j % 3], v);
        }
    }
    if (bounds) {
        for (int d = 0; d < 3; ++d) {
            bounds[d] = lo[d];
            bounds[3 + d] = hi[d];
        }
    }
    return STRO_OK;
}

int stro_sphere_stl(float radius, int32_t segments, int32_t rings, uint8_t* out, size_t cap,
                    size_t* len) {
    if (!len || segments < 3 || rings < 2) return fail(STRO_ERR_INVALID, "bad sphere mesh arguments");
    const float pi = 3.14159265358979323846f;
    auto pt = [&](int i, int j, float p[3]) {
        const float theta = float(j) * pi / float(rings);
        const float phi = float(i) * 2.0f * pi / float(segments);
        p[0] = radius * std::sin(theta) * std::cos(phi);
        p[1] = radius * std::sin(theta) * std::sin(phi);
        p[2] = radius * std::cos(theta);
    };
    const size_t ntri = size_t(segments) * size_t(2 * rings - 2);
    const size_t bytes = 84 + ntri * 50;
    *len = bytes;
    if (!out) return STRO_OK;  // size query
    if (cap < bytes) return fail(STRO_ERR_INVALID, "output buffer too small");
    std::memset(out, 0, 84);
    const uint32_t n32 = uint32_t(ntri);
    std::memcpy(out + 80, &n32, 4);
    uint8_t* w = out + 84;
    auto put = [&](const float* a, const float* b, const float* c) {
        std::memset(w, 0, 50);  // normal (unused) and attribute byte count
        std::memcpy(w + 12, a, 12);
        std::memcpy(w + 24, b, 12);
        std::memcpy(w + 36, c, 12);
        w += 50;
    };
    for (int j = 0; j < rings; ++j)
        for (int i = 0; i < segments; ++i) {
            float a[3], b[3], c[3], d[3];
            pt(i, j, a);
            pt(i + 1, j, b);
            pt(i, j + 1, c);
            pt(i + 1, j + 1, d);
            if (j > 0) put(a, b, c);
            if (j < rings - 1) put(b, d, c);
        }
    return STRO_OK;
}

int stro_mesh_solid_fractions(stro_ctx* ctx, const float* tris, uint32_t ntri, int32_t nx,
                              int32_t ny, int32_t nz, float scale, const float offset[3],
                              float* eps, double* seconds) {
    if (!ctx || !offset || !eps || (ntri > 0 && !tris))
        return fail(STRO_ERR_INVALID, "null argument");
    if (nx < 1 || ny < 1 || nz < 1) return fail(STRO_ERR_INVALID, "lattice dimensions must be >= 1");
    const uint64_t N = uint64_t(nx) * uint64_t(ny) * uint64_t(nz);
    if (N >= (uint64_t(1) << 31)) return fail(STRO_ERR_INVALID, "lattice too large");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    float *d_in = nullptr, *d_t = nullptr, *d_eps = nullptr;
    uint32_t *d_start = nullptr, *d_list = nullptr, *d_cols = nullptr;
    int* d_err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = STRO_OK;
    std::vector<float> t(size_t(ntri) * 9);
    std::vector<uint32_t> start(size_t(ny) * nz + 1, 0), list, busy;
    auto cleanup = [&]() {
        cudaFree(d_in);
        cudaFree(d_t);
        cudaFree(d_eps);
        cudaFree(d_start);
        cudaFree(d_list);
        cudaFree(d_cols);
        cudaFree(d_err);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
#define VX_CUDA(call)                                  \
    do {                                               \
        const cudaError_t e_ = (call);                 \
        if (e_ != cudaSuccess) {                       \
            rc = cuda_fail(e_, #call);                 \
            cleanup();                                 \
            return rc;                                 \
        }                                              \
    } while (0)
    try {
        const size_t tbytes = sizeof(float) * t.size();
        if (ntri > 0) {
            VX_CUDA(cudaMalloc(&d_in, tbytes));
            VX_CUDA(cudaMalloc(&d_t, tbytes));
            VX_CUDA(cudaMemcpyAsync(d_in, tris, tbytes, cudaMemcpyHostToDevice, st));
            const uint32_t nv = ntri * 3;
            k_transform<<<(nv + 255) / 256, 256, 0, st>>>(d_in, d_t, nv, scale, offset[0], offset[1],
                                                          offset[2]);
            VX_CUDA(cudaGetLastError());
            VX_CUDA(cudaMemcpyAsync(t.data(), d_t, tbytes, cudaMemcpyDeviceToHost, st));
            VX_CUDA(cudaStreamSynchronize(st));
        }
        // buckets over (y, z) by the triangle's bounding box widened by half a cell
        std::vector<int> lo(size_t(ntri) * 4);
        for (uint32_t i = 0; i < ntri; ++i) {
            const float* p = &t[9 * size_t(i)];
            const float ymin = std::min(std::min(p[1], p[4]), p[7]);
            const float ymax = std::max(std::max(p[1], p[4]), p[7]);
            const float zmin = std::min(std::min(p[2], p[5]), p[8]);
            const float zmax = std::max(std::max(p[2], p[5]), p[8]);
            const double fy0 = std::floor(double(ymin - 0.5f)), fy1 = std::ceil(double(ymax + 0.5f));
            const double fz0 = std::floor(double(zmin - 0.5f)), fz1 = std::ceil(double(zmax + 0.5f));
            int* b = &lo[4 * size_t(i)];
            b[0] = int(std::max(0.0, std::min(fy0, double(ny))));
            b[1] = int(std::min(double(ny - 1), std::max(fy1, -1.0)));
            b[2] = int(std::max(0.0, std::min(fz0, double(nz))));
            b[3] = int(std::min(double(nz - 1), std::max(fz1, -1.0)));
            if (b[0] > b[1] || b[2] > b[3]) continue;
            for (int z = b[2]; z <= b[3]; ++z)
                for (int y = b[0]; y <= b[1]; ++y) ++start[size_t(z) * ny + y + 1];
        }
        for (size_t c = 1; c < start.size(); ++c) start[c] += start[c - 1];
        list.resize(start.back());
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (uint32_t i = 0; i < ntri; ++i) {
            const int* b = &lo[4 * size_t(i)];
            if (b[0] > b[1] || b[2] > b[3]) continue;
            for (int z = b[2]; z <= b[3]; ++z)
                for (int y = b[0]; y <= b[1]; ++y) list[fill[size_t(z) * ny + y]++] = i;
        }
        for (size_t c = 0; c + 1 < start.size(); ++c)
            if (start[c + 1] > start[c]) busy.push_back(uint32_t(c));
    } catch (const std::bad_alloc&) {
        cleanup();
        return fail(STRO_ERR_OOM, "host allocation failed");
    }
    VX_CUDA(cudaMalloc(&d_eps, sizeof(float) * N));
    VX_CUDA(cudaMalloc(&d_start, sizeof(uint32_t) * start.size()));
    VX_CUDA(cudaMalloc(&d_list, sizeof(uint32_t) * std::max<size_t>(list.size(), 1)));
    VX_CUDA(cudaMalloc(&d_err, sizeof(int)));
    VX_CUDA(cudaMalloc(&d_cols, sizeof(uint32_t) * std::max<size_t>(busy.size(), 1)));
    if (!busy.empty())
        VX_CUDA(cudaMemcpyAsync(d_cols, busy.data(), sizeof(uint32_t) * busy.size(),
                                cudaMemcpyHostToDevice, st));
    VX_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    VX_CUDA(cudaMemsetAsync(d_eps, 0, sizeof(float) * N, st));
    VX_CUDA(cudaMemcpyAsync(d_start, start.data(), sizeof(uint32_t) * start.size(),
                            cudaMemcpyHostToDevice, st));
    if (!list.empty())
        VX_CUDA(cudaMemcpyAsync(d_list, list.data(), sizeof(uint32_t) * list.size(),
                                cudaMemcpyHostToDevice, st));
    VX_CUDA(cudaEventCreate(&e0));
    VX_CUDA(cudaEventCreate(&e1));
    VX_CUDA(cudaEventRecord(e0, st));
    if (!busy.empty()) {
        k_columns<<<uint32_t(busy.size()), 128, 0, st>>>(d_t, d_start, d_list, d_cols, nx, ny,
                                                         d_eps, d_err);
        VX_CUDA(cudaGetLastError());
    }
    VX_CUDA(cudaEventRecord(e1, st));
    int err = 0;
    VX_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    VX_CUDA(cudaMemcpyAsync(eps, d_eps, sizeof(float) * N, cudaMemcpyDeviceToHost, st));
    VX_CUDA(cudaStreamSynchronize(st));
    float ms = 0.0f;
    VX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (seconds) *seconds = double(ms) * 1e-3;
#undef VX_CUDA
    cleanup();
    if (err != 0)
        return fail(STRO_ERR_INVALID, "a sub-ray crosses the mesh more than 128 times");
    return STRO_OK;
}

}  // extern "C"
