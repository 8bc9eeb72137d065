// Field initialisation, moments and fixed-order FP64 reductions.
//
// initField restates Kernels.metal:393-453 (trigonometric values are taken in
// double precision and rounded to FP32, so the initial state does not depend
// on a device math library). momentsEven restates Kernels.metal:359-380. The
// reductions (kinetic energy, dissipation, mass, non-finite count) accumulate
// FP64 per thread in a fixed cell order, reduce each block with a fixed
// shuffle tree and fold the block partials in a second fixed-order pass: the
// result is bitwise reproducible run to run (no atomics).
#include "lbm_device.cuh"
#include "lbm_launch.h"

namespace stro {

namespace {

constexpr int kThreads = 256;

template <typename S>
__device__ __forceinline__ void load_cell(const FieldView& v, uint32_t n, float (&fh)[19]) {
    const S* f = static_cast<const S*>(v.f);
    sfor<0, 19>([&](auto I) { fh[I] = load_ddf<S>(f + uint64_t(I) * v.plane + n); });
}

// Moments of one cell after an even step count, as momentsEven computes them.
__device__ __forceinline__ void cell_moments(const FieldView& v, uint32_t n, const float (&fh)[19],
                                             float& rhom1, float& rho, float& ux, float& uy,
                                             float& uz) {
    rhom1 = fh[0];
    sfor<1, 19>([&](auto I) { rhom1 += fh[I]; });
    float px = fh[1], py = fh[3], pz = fh[5];
    sfor<2, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcx(i) > 0) px += fh[i];
        if constexpr (dcx(i) < 0) px -= fh[i];
    });
    sfor<4, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcy(i) > 0) py += fh[i];
        if constexpr (dcy(i) < 0) py -= fh[i];
    });
    sfor<6, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcz(i) > 0) pz += fh[i];
        if constexpr (dcz(i) < 0) pz -= fh[i];
    });
    float Fx = v.fx, Fy = v.fy, Fz = v.fz;
    if (v.ffield != nullptr) {
        Fx = v.fx + v.ffield[n];
        Fy = v.fy + v.ffield[uint64_t(v.N) + n];
        Fz = v.fz + v.ffield[2ull * v.N + n];
    }
    rho = 1.0f + rhom1;
    ux = (px + 0.5f * Fx) / rho;
    uy = (py + 0.5f * Fy) / rho;
    uz = (pz + 0.5f * Fz) / rho;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_init_field(FieldView v, uint32_t mode, float A,
                                                         float tau) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= v.N) return;
    float ux = 0.f, uy = 0.f, uz = 0.f, sxx = 0.f, sxz = 0.f, syz = 0.f, rhom1 = 0.f;
    const uint32_t x = n % v.nx, t = n / v.nx, y = t % v.ny, z = t / v.ny;
    const float pi = 3.14159265358979323846f;
    auto S_ = [](float a) { return (float)sin((double)a); };
    auto C_ = [](float a) { return (float)cos((double)a); };
    if (mode == 1u) {
        const float kx = 2.0f * pi / (float)v.nx, ky = 2.0f * pi / (float)v.ny;
        const float xa = (float)x + 0.5f, ya = (float)y + 0.5f;
        ux = A * S_(kx * xa) * C_(ky * ya);
        uy = -A * C_(kx * xa) * S_(ky * ya);
        sxx = A * kx * C_(kx * xa) * C_(ky * ya);
        rhom1 = 0.75f * A * A * (C_(2.0f * kx * xa) + C_(2.0f * ky * ya));
    }
    if (mode == 2u) {
        const float kx = 2.0f * pi / (float)v.nx, ky = 2.0f * pi / (float)v.ny,
                    kz = 2.0f * pi / (float)v.nz;
        const float xa = kx * ((float)x + 0.5f), ya = ky * ((float)y + 0.5f),
                    za = kz * ((float)z + 0.5f);
        ux = A * S_(xa) * C_(ya) * C_(za);
        uy = -A * C_(xa) * S_(ya) * C_(za);
        sxx = A * kx * C_(xa) * C_(ya) * C_(za);
        sxz = -0.5f * A * kz * S_(xa) * C_(ya) * S_(za);
        syz = 0.5f * A * kz * C_(xa) * S_(ya) * S_(za);
        rhom1 = 0.1875f * A * A * (C_(2.0f * xa) + C_(2.0f * ya)) * (C_(2.0f * za) + 2.0f);
    }
    const float rho = 1.0f + rhom1;
    const float u2 = ux * ux + uy * uy + uz * uz;
    S* f = static_cast<S*>(v.f);
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const float cu = 3.0f * ((float)dcx(i) * ux + (float)dcy(i) * uy + (float)dcz(i) * uz);
        const float feq = wgt(i) * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
        const float cc = (float)(dcx(i) * dcx(i) - dcy(i) * dcy(i));
        const float scc = sxx * cc + 2.0f * sxz * (float)(dcx(i) * dcz(i)) +
                          2.0f * syz * (float)(dcy(i) * dcz(i));
        const float fneq = -3.0f * wgt(i) * tau * scc;
        store_ddf<S>(f + uint64_t(i) * v.plane + n, feq + fneq);
    });
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_moments(FieldView v, float4* out) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= v.N) return;
    if (v.cell != nullptr && (v.cell[n] & CELL_TYPE_MASK) != CELL_FLUID) {
        out[n] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    float fh[19];
    load_cell<S>(v, n, fh);
    float rhom1, rho, ux, uy, uz;
    cell_moments(v, n, fh, rhom1, rho, ux, uy, uz);
    out[n] = make_float4(ux, uy, uz, rho);
}

// The |u| colormap of one z slice (colorize + speedColor, Kernels.metal:465-500)
// fused with momentsEven: the velocity is formed from the slice's own DDFs
// exactly as k_moments forms it, so the image equals colorize applied to the
// moments probe. Walls and cells with eps >= 0.5 are slate; other cells take
// the four-stop map of clamp(|u| / uref, 0, 1) and, for 0 < eps < 0.5, a blend
// toward slate by eps (the half-vector mix evaluated in float and rounded
// once). out: nx*ny RGBA binary16 texels, row y at ny-1-y as the reference's
// texture write.
template <typename S>
__global__ void k_render(FieldView v, const float* eps, uint32_t z, float uref, __half* out) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= v.nx || y >= v.ny) return;
    const uint32_t n = (z * v.ny + y) * v.nx + x;
    const uint8_t flag = v.cell != nullptr ? (v.cell[n] & CELL_TYPE_MASK) : CELL_FLUID;
    const float e = eps != nullptr ? eps[n] : 0.0f;
    const __half slate[3] = {__float2half_rn(0.30f), __float2half_rn(0.28f), __float2half_rn(0.25f)};
    __half rgb[3];
    if (flag != CELL_FLUID || e >= 0.5f) {
        rgb[0] = slate[0]; rgb[1] = slate[1]; rgb[2] = slate[2];
    } else {
        float fh[19];
        load_cell<S>(v, n, fh);
        float rhom1, rho, ux, uy, uz;
        cell_moments(v, n, fh, rhom1, rho, ux, uy, uz);
        const float len = sqrtf(ux * ux + uy * uy + uz * uz);
        const float s = fminf(fmaxf(len / uref, 0.0f), 1.0f);
        // ember map: charcoal -> deep red -> orange -> pale amber
        const float c0[3] = {(float)0.055, (float)0.045, (float)0.040};
        const float c1[3] = {(float)0.420, (float)0.100, (float)0.050};
        const float c2[3] = {(float)0.900, (float)0.450, (float)0.100};
        const float c3[3] = {(float)1.000, (float)0.930, (float)0.780};
        const float* a;
        const float* b;
        float t;
        if (s < 0.35f) { a = c0; b = c1; t = s / 0.35f; }
        else if (s < 0.70f) { a = c1; b = c2; t = (s - 0.35f) / 0.35f; }
        else { a = c2; b = c3; t = (s - 0.70f) / 0.30f; }
        for (int k = 0; k < 3; ++k) rgb[k] = __float2half_rn(a[k] + (b[k] - a[k]) * t);
        if (e > 0.0f) {
            const float te = __half2float(__float2half_rn(e));
            for (int k = 0; k < 3; ++k) {
                const float c = __half2float(rgb[k]);
                rgb[k] = __float2half_rn(c + (__half2float(slate[k]) - c) * te);
            }
        }
    }
    __half* px = out + 4 * (size_t(v.ny - 1 - y) * v.nx + x);
    px[0] = rgb[0];
    px[1] = rgb[1];
    px[2] = rgb[2];
    px[3] = __float2half_rn(1.0f);
}

// Per cell: |u|^2 (FP32, as the host energy loop forms it) and the viscous
// dissipation 2 nu S:S with S = -(3 omega / (2 rho)) Pi_neq, both formed in
// FP32 and summed in FP64 (one FP64 add per cell and quantity: the FP64 rate
// of this part is a small fraction of its FP32 rate, so per-cell FP64
// arithmetic would make the reduction compute-bound). nu comes from the host,
// formed in FP64 from omega.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_observables(FieldView v, float omega, float nu,
                                                          double* partials) {
    double acc[2] = {0.0, 0.0};
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N; n += gridDim.x * blockDim.x) {
        if (v.cell != nullptr && (v.cell[n] & CELL_TYPE_MASK) != CELL_FLUID) continue;
        float fh[19];
        load_cell<S>(v, n, fh);
        float rhom1, rho, ux, uy, uz;
        cell_moments(v, n, fh, rhom1, rho, ux, uy, uz);
        const float u2 = ux * ux + uy * uy + uz * uz;
        acc[0] += (double)u2;
        float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            const float cu = 3.0f * cdot<i>(ux, uy, uz);
            const float feq = wgt(i) * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
            const float d = fh[i] - feq;
            if constexpr (dcx(i) != 0) pxx += d;
            if constexpr (dcy(i) != 0) pyy += d;
            if constexpr (dcz(i) != 0) pzz += d;
            if constexpr (dcx(i) * dcy(i) > 0) pxy += d;
            if constexpr (dcx(i) * dcy(i) < 0) pxy -= d;
            if constexpr (dcx(i) * dcz(i) > 0) pxz += d;
            if constexpr (dcx(i) * dcz(i) < 0) pxz -= d;
            if constexpr (dcy(i) * dcz(i) > 0) pyz += d;
            if constexpr (dcy(i) * dcz(i) < 0) pyz -= d;
        });
        const float pipi = pxx * pxx + pyy * pyy + pzz * pzz +
                           2.0f * (pxy * pxy + pxz * pxz + pyz * pyz);
        const float s = 1.5f * omega / rho;
        acc[1] += (double)(2.0f * nu * s * s * pipi);
    }
    block_reduce_store<2>(acc, partials + 2u * blockIdx.x);
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_mass(FieldView v, double* partials) {
    double acc[1] = {0.0};
    const S* f = static_cast<const S*>(v.f);
    for (int i = 0; i < 19; ++i)
        for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N;
             n += gridDim.x * blockDim.x)
            acc[0] += (double)load_ddf<S>(f + uint64_t(i) * v.plane + n);
    block_reduce_store<1>(acc, partials + blockIdx.x);
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_nonfinite(FieldView v, double* partials) {
    double acc[1] = {0.0};
    const S* f = static_cast<const S*>(v.f);
    for (int i = 0; i < 19; ++i)
        for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N;
             n += gridDim.x * blockDim.x)
            if (!isfinite(load_ddf<S>(f + uint64_t(i) * v.plane + n))) acc[0] += 1.0;
    block_reduce_store<1>(acc, partials + blockIdx.x);
}

template <int K>
__global__ void __launch_bounds__(kThreads) k_fold(const double* partials, int nblocks,
                                                   double* out) {
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += partials[b * K + k];
    block_reduce_store<K>(acc, out);
}

}  // namespace

int reduction_blocks(uint64_t count) {
    uint64_t b = (count + 1023) / 1024;
    if (b < 1) b = 1;
    if (b > uint64_t(kReductionMaxBlocks)) b = kReductionMaxBlocks;
    return int(b);
}

cudaError_t launch_fold(const double* partials, int nblocks, int K, double* out, cudaStream_t st) {
    switch (K) {
        case 1: k_fold<1><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        case 2: k_fold<2><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        case 3: k_fold<3><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_init_field(const FieldView& v, int half_storage, uint32_t mode, float amplitude,
                              float tau, cudaStream_t st) {
    const unsigned grid = (v.N + kThreads - 1) / kThreads;
    if (half_storage) k_init_field<__half><<<grid, kThreads, 0, st>>>(v, mode, amplitude, tau);
    else k_init_field<float><<<grid, kThreads, 0, st>>>(v, mode, amplitude, tau);
    return cudaGetLastError();
}

cudaError_t launch_moments(const FieldView& v, int half_storage, float4* out, cudaStream_t st) {
    const unsigned grid = (v.N + kThreads - 1) / kThreads;
    if (half_storage) k_moments<__half><<<grid, kThreads, 0, st>>>(v, out);
    else k_moments<float><<<grid, kThreads, 0, st>>>(v, out);
    return cudaGetLastError();
}

cudaError_t launch_render(const FieldView& v, int half_storage, const float* eps, uint32_t z,
                          float uref, __half* out, cudaStream_t st) {
    const dim3 block(32, 8);
    const dim3 grid((v.nx + 31) / 32, (v.ny + 7) / 8);
    if (half_storage) k_render<__half><<<grid, block, 0, st>>>(v, eps, z, uref, out);
    else k_render<float><<<grid, block, 0, st>>>(v, eps, z, uref, out);
    return cudaGetLastError();
}

cudaError_t launch_observables(const FieldView& v, int half_storage, float omega,
                               double* partials, double* out, cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    const float nu = float((1.0 / double(omega) - 0.5) / 3.0);
    if (half_storage) k_observables<__half><<<nb, kThreads, 0, st>>>(v, omega, nu, partials);
    else k_observables<float><<<nb, kThreads, 0, st>>>(v, omega, nu, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 2, out, st);
}

cudaError_t launch_mass(const FieldView& v, int half_storage, double* partials, double* out,
                        cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    if (half_storage) k_mass<__half><<<nb, kThreads, 0, st>>>(v, partials);
    else k_mass<float><<<nb, kThreads, 0, st>>>(v, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 1, out, st);
}

cudaError_t launch_nonfinite(const FieldView& v, int half_storage, double* partials, double* out,
                             cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    if (half_storage) k_nonfinite<__half><<<nb, kThreads, 0, st>>>(v, partials);
    else k_nonfinite<float><<<nb, kThreads, 0, st>>>(v, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 1, out, st);
}

}  // namespace stro

// ---------------------------------------------------------------------------
// Allocation-free observables for callers that cannot allocate device memory.
//
// Some hosts of this library must not call cudaMalloc while they step a
// lattice. One example is a framework whose caching allocator already owns
// the HBM. Another is a real-time loop, where cudaMalloc may synchronise the
// device and stall the loop. A third is code that runs while a stream is
// being captured. Such callers hold the DDF state in memory they own and want
// the kinetic-energy and dissipation sums of it. stro_observables_noalloc runs
// the same reduction kernels as stro_sim_kinetic_energy / stro_sim_dissipation
// and allocates nothing itself. Its per-block partial sums go to the
// file-scope array below. The module holds that array on every GPU that loads
// the library, until the process exits.
#include <mutex>

#include "runtime_internal.h"

namespace {

// The most blocks reduction_blocks() ever uses, so every lattice it accepts fits.
constexpr int kNoAllocMaxBlocks = stro::kReductionMaxBlocks;
static_assert(kNoAllocMaxBlocks * 2 * sizeof(double) <= 32 * 1024,
              "the allocation-free scratch array is stated as 32 KB");
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks * 2];  // 32 KB

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the host-side symbol is only a stand-in, not a device address).
int noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return stro::rt::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return stro::rt::fail(STRO_ERR_INVALID, "device index beyond the scratch table");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return stro::rt::cuda_fail(e, "cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<double*>(g_noalloc_ptr[dev]);
    return STRO_OK;
}

}  // namespace

extern "C" int stro_observables_noalloc(const void* f, int32_t precision, int32_t nx, int32_t ny,
                                        int32_t nz, uint64_t plane_stride,
                                        const uint8_t* cell_types, float omega,
                                        const float force[3], double* out, void* stream) {
    using stro::rt::fail;
    if (!f || !out) return fail(STRO_ERR_INVALID, "state and output pointers are required");
    if (precision != STRO_FP32 && precision != STRO_FP16S)
        return fail(STRO_ERR_INVALID, "precision must be STRO_FP32 or STRO_FP16S");
    if (nx < 1 || ny < 1 || nz < 1) return fail(STRO_ERR_INVALID, "lattice dimensions must be >= 1");
    const uint64_t N = uint64_t(nx) * uint64_t(ny) * uint64_t(nz);
    if (N >= (1ull << 31)) return fail(STRO_ERR_INVALID, "lattice too large (N must be < 2^31 cells)");
    if (plane_stride < N) return fail(STRO_ERR_INVALID, "plane stride must be at least nx*ny*nz");
    if (!(omega > 0.0f && omega < 2.0f))  // also refuses NaN
        return fail(STRO_ERR_INVALID, "omega must be finite and in (0, 2)");
    const int nb = stro::reduction_blocks(N);
    if (nb > kNoAllocMaxBlocks)
        return fail(STRO_ERR_INVALID, "reduction needs more partials than the scratch array holds");
    double* scratch = nullptr;
    const int rc = noalloc_scratch(&scratch);
    if (rc != STRO_OK) return rc;
    stro::FieldView v{};
    v.f = const_cast<void*>(f);
    v.plane = plane_stride;
    v.nx = uint32_t(nx); v.ny = uint32_t(ny); v.nz = uint32_t(nz);
    v.N = uint32_t(N);
    v.cell = cell_types;
    v.ffield = nullptr;
    v.fx = force ? force[0] : 0.0f;
    v.fy = force ? force[1] : 0.0f;
    v.fz = force ? force[2] : 0.0f;
    // Every block writes its own partials before the fold reads them, so nothing in
    // the scratch array has to start at zero; what a previous call left there is
    // simply overwritten.
    const cudaError_t e = stro::launch_observables(v, precision == STRO_FP16S, omega, scratch, out,
                                                   static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return stro::rt::cuda_fail(e, "observables launch");
    return STRO_OK;
}
