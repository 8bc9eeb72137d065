// Compiles the reference's unmodified Sources/StrouhalCore/Kernels.metal as
// C++ (through ref_shim/metal_stdlib) twice — FPXX=float and FPXX=half — and
// exports C entry points that run one kernel over every thread index n in
// order, the way a Metal dispatch of N threads would.
//
// Test infrastructure only: the oracle restatement in lbm_oracle.cpp is
// checked against these entry points value-for-value. Built by
// oracle/build_oracle.py into oracle/_ref/ (never committed); the kernel source is
// read from the reference tree at build time, not copied.
#include <metal_stdlib>
#include <cstddef>
#include <cstdint>

namespace ref_f32 {
#define FPXX float
#include "Kernels.metal"
#undef FPXX
}  // namespace ref_f32

namespace ref_f16 {
#define FPXX half
#include "Kernels.metal"
#undef FPXX
}  // namespace ref_f16

static_assert(sizeof(ref_f32::Params) == 80, "Params is 20 x 4 B (Kernels.metal:49-63)");
static_assert(sizeof(ref_f32::InitParams) == 32, "InitParams is 8 x 4 B (Kernels.metal:386-391)");
static_assert(sizeof(ref_f32::VizParams) == 32, "VizParams is 8 x 4 B (Kernels.metal:458-463)");
static_assert(sizeof(metal::half4) == 8, "half4 is four binary16 values");

extern "C" {

// One full `step` dispatch (Kernels.metal:230-355) over n = 0..N-1.
// half_storage selects the FPXX=half build; f points at 19*N values of that type.
int ref_step(int half_storage, void* f, const uint8_t* flags, const uint32_t* solid_mask,
             const uint32_t* lid_mask, const void* params, float* force4, const float* eps) {
    if (half_storage) {
        const auto& p = *static_cast<const ref_f16::Params*>(params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n)
            ref_f16::step(static_cast<metal::half*>(f), flags, solid_mask, lid_mask, p,
                          reinterpret_cast<metal::float4*>(force4), eps, n);
    } else {
        const auto& p = *static_cast<const ref_f32::Params*>(params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n)
            ref_f32::step(static_cast<float*>(f), flags, solid_mask, lid_mask, p,
                          reinterpret_cast<metal::float4*>(force4), eps, n);
    }
    return 0;
}

// One `momentsEven` dispatch (Kernels.metal:359-380); out holds N float4.
int ref_moments(int half_storage, const void* f, const uint8_t* flags, const void* params,
                float* out4) {
    if (half_storage) {
        const auto& p = *static_cast<const ref_f16::Params*>(params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n)
            ref_f16::momentsEven(static_cast<const metal::half*>(f), flags,
                                 reinterpret_cast<metal::float4*>(out4), p, n);
    } else {
        const auto& p = *static_cast<const ref_f32::Params*>(params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n)
            ref_f32::momentsEven(static_cast<const float*>(f), flags,
                                 reinterpret_cast<metal::float4*>(out4), p, n);
    }
    return 0;
}

// One `initField` dispatch (Kernels.metal:393-453). init_params is the
// 32-byte InitParams {nx, ny, nz, mode, amplitude, tau, pad, pad}.
int ref_init_field(int half_storage, void* f, const void* init_params) {
    if (half_storage) {
        const auto& p = *static_cast<const ref_f16::InitParams*>(init_params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n) ref_f16::initField(static_cast<metal::half*>(f), p, n);
    } else {
        const auto& p = *static_cast<const ref_f32::InitParams*>(init_params);
        const uint32_t N = p.nx * p.ny * p.nz;
        for (uint32_t n = 0; n < N; ++n) ref_f32::initField(static_cast<float*>(f), p, n);
    }
    return 0;
}

// One `colorize` dispatch (Kernels.metal:476-500) over gid in [0,nx) x [0,ny):
// moments4 holds N float4 (momentsEven output), viz_params is the 32-byte
// VizParams {nx, ny, nz, zSlice, uref, useEps, pad, pad}, out receives the
// nx*ny half4 image (y flipped as the kernel writes it).
int ref_colorize(const float* moments4, const uint8_t* flags, const float* eps,
                 const void* viz_params, uint16_t* out_half4) {
    const auto& v = *static_cast<const ref_f32::VizParams*>(viz_params);
    metal::texture2d<metal::half, metal::access::write> tex;
    tex.data = reinterpret_cast<metal::half4*>(out_half4);
    tex.width = v.nx;
    for (uint32_t y = 0; y < v.ny; ++y)
        for (uint32_t x = 0; x < v.nx; ++x)
            ref_f32::colorize(reinterpret_cast<const metal::float4*>(moments4), flags, eps, v, tex,
                              metal::uint2(x, y));
    return 0;
}

}  // extern "C"
