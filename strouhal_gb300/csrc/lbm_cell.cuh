// Per-cell bodies of the D3Q19 AA step, shared by the single-lattice kernels
// (lbm_step.cu) and the batched persistent kernel (lbm_batch.cu).
//
// Restates the reference's `collide` (Kernels.metal:105-228) and the two
// branches of its `step` kernel (Kernels.metal:252-354) with the same FP32
// operation order; see lbm_step.cu for the arithmetic contract.
#pragma once

#include "lbm_device.cuh"

namespace stro {

__device__ __forceinline__ int wrapi(int v, int n) {  // Kernels.metal:73-77
    v += (v < 0) ? n : 0;
    v -= (v >= n) ? n : 0;
    return v;
}

// Ramped moving-wall velocities of one step (Sim.swift:270-275).
struct WallVel {
    float uin, lx, ly, lz;
    __device__ __forceinline__ explicit WallVel(const StepArgs& a)
        : uin(a.uin), lx(a.ulid_x), ly(a.ulid_y), lz(a.ulid_z) {}
    __device__ __forceinline__ WallVel(float u, float x, float y, float z)
        : uin(u), lx(x), ly(y), lz(z) {}
};

// Wall velocity of a moving-wall cell at row wy, Kernels.metal:79-87.
__device__ __forceinline__ void wall_velocity(uint8_t wf, int wy, const StepArgs& a,
                                              const WallVel& wv, float& ux, float& uy,
                                              float& uz) {
    if (wf == CELL_LID) {
        ux = wv.lx; uy = wv.ly; uz = wv.lz;
        return;
    }
    uy = 0.0f; uz = 0.0f;
    if (a.inflow_uniform != 0) { ux = wv.uin; return; }
    const float H = (float)a.ny - 2.0f;
    const float yd = (float)wy - 0.5f;
    ux = fmaxf(4.0f * wv.uin * yd * (H - yd) / (H * H), 0.0f);
}

// Relaxation of the rest direction and the nine antipodal pairs
// (Kernels.metal:169-227). FORCE adds the TRT-split Guo source, NT blends with
// the Noble-Torczynski bounce operator and accumulates its force.
template <bool FORCE, bool NT>
__device__ __forceinline__ void relax(float (&fh)[19], float wp, float wm, float rho, float rhom1,
                                      float ux, float uy, float uz, float u2, float Fx, float Fy,
                                      float Fz, float eps, float& ntx, float& nty, float& ntz) {
    const float feq0 = wgt(0) * (rhom1 - 1.5f * rho * u2);
    float uF = 0.0f, ap = 0.0f, am = 0.0f;
    if constexpr (FORCE) {
        uF = ux * Fx + uy * Fy + uz * Fz;
        ap = 1.0f - 0.5f * wp;
        am = 1.0f - 0.5f * wm;
    }
    float B = 0.0f, omb = 1.0f;
    if constexpr (!NT) {
        if constexpr (FORCE) {
            const float s0 = wgt(0) * ap * (-3.0f * uF);
            fh[0] = fmaf(wp, feq0 - fh[0], fh[0]) + s0;
        } else {
            fh[0] = fmaf(wp, feq0 - fh[0], fh[0]);
        }
    } else {
        const float tw = 1.0f / wp - 0.5f;
        B = eps * tw / ((1.0f - eps) + tw);
        omb = 1.0f - B;
        if constexpr (FORCE) {
            const float s0 = wgt(0) * ap * (-3.0f * uF);
            fh[0] += omb * (wp * (feq0 - fh[0]) + s0);
        } else {
            fh[0] += omb * (wp * (feq0 - fh[0]));
        }
    }
    const float u2t = 1.5f * u2;
    sfor<0, 9>([&](auto P) {
        constexpr int i = 2 * P + 1;
        constexpr float w = wgt(i);
        const float cu = 3.0f * cdot<i>(ux, uy, uz);
        const float feqp = w * (rhom1 + rho * (0.5f * cu * cu - u2t));
        const float feqm = w * rho * cu;
        const float fp = 0.5f * (fh[i] + fh[i + 1]);
        const float fm = 0.5f * (fh[i] - fh[i + 1]);
        const float dp = wp * (feqp - fp);
        const float dm = wm * (feqm - fm);
        float up, um;
        if constexpr (FORCE) {
            const float cF = cdot<i>(Fx, Fy, Fz);
            const float sm = w * am * (3.0f * cF);
            const float sp = w * ap * (3.0f * cu * cF - 3.0f * uF);
            up = dp + dm + sp + sm;
            um = dp - dm + sp - sm;
        } else {
            up = dp + dm;
            um = dp - dm;
        }
        if constexpr (!NT) {
            fh[i] += up;
            fh[i + 1] += um;
        } else {
            const float bounce = B * (fh[i + 1] - fh[i]);
            fh[i] += omb * up + bounce;
            fh[i + 1] += omb * um - bounce;
            if constexpr (dcx(i) > 0) ntx -= 2.0f * bounce;
            if constexpr (dcx(i) < 0) ntx += 2.0f * bounce;
            if constexpr (dcy(i) > 0) nty -= 2.0f * bounce;
            if constexpr (dcy(i) < 0) nty += 2.0f * bounce;
            if constexpr (dcz(i) > 0) ntz -= 2.0f * bounce;
            if constexpr (dcz(i) < 0) ntz += 2.0f * bounce;
        }
    });
}

// Relaxation in the fused arithmetic (ARITH_FUSED): the same collision as
// relax() written with fused multiply-adds and shared per-weight products:
//   feq+ = fma(w rho, fma(4.5 cd, cd, -1.5 u2), w (rho-1)),  feq- = (w rho)(3 cd)
//   A = fma(-1/2, f_i + f_j, feq+),  B = fma(-1/2, f_i - f_j, feq-)
//   f_i' = fma(w+, A, fma(w-, B, f_i)),  f_j' = fma(w+, A, fma(-w-, B, f_j))
// with cd = c_i . u, j = opp(i). Equal to relax() in exact arithmetic; the
// oracle evaluates the identical operation sequence (orc kinds 3 and 4).
template <bool FORCE, bool NT>
__device__ __forceinline__ void relax_fused(float (&fh)[19], float wp, float wm, float rho,
                                            float rhom1, float ux, float uy, float uz, float u2,
                                            float Fx, float Fy, float Fz, float eps, float& ntx,
                                            float& nty, float& ntz) {
    const float u2t = 1.5f * u2;
    const float wr0 = wgt(0) * rho, wm0 = wgt(0) * rhom1;
    const float wrs = wgt(1) * rho, wms = wgt(1) * rhom1;
    const float wrl = wgt(7) * rho, wml = wgt(7) * rhom1;
    const float feq0 = fmaf(-wr0, u2t, wm0);
    float uF = 0.0f, ap = 0.0f, am = 0.0f, aps = 0.0f, apl = 0.0f, ams = 0.0f, aml = 0.0f;
    if constexpr (FORCE) {
        uF = fmaf(uz, Fz, fmaf(uy, Fy, ux * Fx));
        ap = fmaf(-0.5f, wp, 1.0f);
        am = fmaf(-0.5f, wm, 1.0f);
        aps = wgt(1) * ap; apl = wgt(7) * ap;
        ams = wgt(1) * am; aml = wgt(7) * am;
    }
    float B = 0.0f, omb = 1.0f;
    if constexpr (!NT) {
        if constexpr (FORCE) {
            const float s0 = wgt(0) * ap * (-3.0f * uF);
            fh[0] = fmaf(wp, feq0 - fh[0], fh[0]) + s0;
        } else {
            fh[0] = fmaf(wp, feq0 - fh[0], fh[0]);
        }
    } else {
        const float tw = 1.0f / wp - 0.5f;
        B = eps * tw / ((1.0f - eps) + tw);
        omb = 1.0f - B;
        if constexpr (FORCE) {
            const float s0 = wgt(0) * ap * (-3.0f * uF);
            fh[0] = fmaf(omb, fmaf(wp, feq0 - fh[0], s0), fh[0]);
        } else {
            fh[0] = fmaf(omb, wp * (feq0 - fh[0]), fh[0]);
        }
    }
    sfor<0, 9>([&](auto P) {
        constexpr int i = 2 * P + 1;
        constexpr bool lng = i >= 7;
        const float wr = lng ? wrl : wrs, wmr = lng ? wml : wms;
        const float cd = cdot<i>(ux, uy, uz);
        const float X = fmaf(4.5f * cd, cd, -u2t);
        const float feqp = fmaf(wr, X, wmr);
        const float feqm = wr * (3.0f * cd);
        const float A = fmaf(-0.5f, fh[i] + fh[i + 1], feqp);
        const float Bm = fmaf(-0.5f, fh[i] - fh[i + 1], feqm);
        float spp = 0.0f, spm = 0.0f;
        if constexpr (FORCE) {
            const float cF = cdot<i>(Fx, Fy, Fz);
            const float sm = (lng ? aml : ams) * (3.0f * cF);
            const float sp = (lng ? apl : aps) * (3.0f * fmaf(3.0f * cd, cF, -uF));
            spp = sp + sm;
            spm = sp - sm;
        }
        if constexpr (!NT) {
            if constexpr (FORCE) {
                fh[i] = fmaf(wp, A, fmaf(wm, Bm, fh[i] + spp));
                fh[i + 1] = fmaf(wp, A, fmaf(-wm, Bm, fh[i + 1] + spm));
            } else {
                fh[i] = fmaf(wp, A, fmaf(wm, Bm, fh[i]));
                fh[i + 1] = fmaf(wp, A, fmaf(-wm, Bm, fh[i + 1]));
            }
        } else {
            const float up = fmaf(wp, A, FORCE ? fmaf(wm, Bm, spp) : wm * Bm);
            const float um = fmaf(wp, A, FORCE ? fmaf(-wm, Bm, spm) : -(wm * Bm));
            const float bounce = B * (fh[i + 1] - fh[i]);
            fh[i] = fmaf(omb, up, bounce) + fh[i];
            fh[i + 1] = fmaf(omb, um, -bounce) + fh[i + 1];
            if constexpr (dcx(i) > 0) ntx -= 2.0f * bounce;
            if constexpr (dcx(i) < 0) ntx += 2.0f * bounce;
            if constexpr (dcy(i) > 0) nty -= 2.0f * bounce;
            if constexpr (dcy(i) < 0) nty += 2.0f * bounce;
            if constexpr (dcz(i) > 0) ntz -= 2.0f * bounce;
            if constexpr (dcz(i) < 0) ntz += 2.0f * bounce;
        }
    });
}

// Arithmetic of the step: ARITH_REFERENCE evaluates the reference's
// expressions as written (value-identical to Kernels.metal in FP32);
// ARITH_FUSED keeps the moments' summation order and evaluates the velocity,
// |u|^2 and the relaxation with fused multiply-adds and shared weight
// products (fewer instructions, rounding differs at the last-bit level).
constexpr int ARITH_REFERENCE = 0;
constexpr int ARITH_FUSED = 1;

// KBC collision (Karlin, Boesch, Chikatamarla, PRE 90, 031302, 2014), an
// extension with no reference counterpart (the reference names a cumulant or
// KBC operator as its roadmap for the transitional Taylor-Green vortex). The
// non-equilibrium part f - feq = ds + dh splits into a shear part ds, the
// Hermite projection of the deviatoric non-equilibrium stress D,
//     ds_i = 4.5 w_i (c_i . D . c_i),
// and the rest dh. ds relaxes at omega, dh at gamma * omega / 2 with the
// entropic stabiliser
//     gamma = 1/beta - (2 - 1/beta) <ds|dh> / <dh|dh>,  beta = omega / 2,
// <x|y> = sum_i x_i y_i / feq_i (raw feq); gamma = 2 is BGK. gamma is kept in
// [0, 2/beta] (the rest relaxes at a rate between 0 and 2): where dh is at the
// rounding level the ratio is noise, and the bound keeps gamma * dh there too.
// With a force,
// u = (p + F/2) / rho leaves f - feq a first moment -F/2; its part
// dk_i = -1.5 w_i (c_i . F) relaxes at omega (as in BGK) and is kept out of
// dh, and the Guo source (1 - omega/2) w_i (3 c.F + 9 (c.u)(c.F) - 3 u.F) is
// added, so the momentum changes by F exactly as with BGK + Guo. The per-
// direction values are recomputed in each pass instead of held in registers.
template <int I>
__device__ __forceinline__ float kbc_geq(float rho, float rhom1, float ux, float uy, float uz,
                                         float u2) {
    const float cu = I == 0 ? 0.0f : 3.0f * cdot<I>(ux, uy, uz);
    return wgt(I) * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
}

// c_i . D . c_i: the diagonal terms in x, y, z order, then twice the one
// off-diagonal term of a two-component direction.
template <int I>
__device__ __forceinline__ float kbc_cdc(float dxx, float dyy, float dzz, float dxy, float dxz,
                                         float dyz) {
    constexpr int a = dcx(I), b = dcy(I), c = dcz(I);
    if constexpr (I == 0) {
        return 0.0f;
    } else if constexpr (a != 0 && b != 0) {
        return (dxx + dyy) + 2.0f * (a * b > 0 ? dxy : -dxy);
    } else if constexpr (a != 0 && c != 0) {
        return (dxx + dzz) + 2.0f * (a * c > 0 ? dxz : -dxz);
    } else if constexpr (b != 0 && c != 0) {
        return (dyy + dzz) + 2.0f * (b * c > 0 ? dyz : -dyz);
    } else {
        return a != 0 ? dxx : (b != 0 ? dyy : dzz);
    }
}

template <bool FORCE>
__device__ __forceinline__ void relax_kbc(float (&fh)[19], float w, float rho, float rhom1,
                                          float ux, float uy, float uz, float u2, float Fx,
                                          float Fy, float Fz) {
    float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        const float d = fh[i] - kbc_geq<i>(rho, rhom1, ux, uy, uz, u2);
        if constexpr (dcx(i) != 0) pxx = (i == 1) ? d : pxx + d;
        if constexpr (dcy(i) != 0) pyy = (i == 3) ? d : pyy + d;
        if constexpr (dcz(i) != 0) pzz = (i == 5) ? d : pzz + d;
        if constexpr (dcx(i) * dcy(i) > 0) pxy = (i == 7) ? d : pxy + d;
        if constexpr (dcx(i) * dcy(i) < 0) pxy -= d;
        if constexpr (dcx(i) * dcz(i) > 0) pxz = (i == 11) ? d : pxz + d;
        if constexpr (dcx(i) * dcz(i) < 0) pxz -= d;
        if constexpr (dcy(i) * dcz(i) > 0) pyz = (i == 15) ? d : pyz + d;
        if constexpr (dcy(i) * dcz(i) < 0) pyz -= d;
    });
    const float tr = (pxx + pyy + pzz) * (1.0f / 3.0f);
    const float dxx = pxx - tr, dyy = pyy - tr, dzz = pzz - tr;
    // dh of direction i (ds and, with a force, dk taken out)
    auto kbc_dh = [&](auto I, float geq, float ds) {
        constexpr int i = I;
        float dh = (fh[i] - geq) - ds;
        if constexpr (FORCE) {
            const float dk = i == 0 ? 0.0f : (-1.5f * wgt(i)) * cdot<i>(Fx, Fy, Fz);
            dh = dh - dk;
        }
        return dh;
    };
    float sh = 0.0f, hh = 0.0f;
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const float geq = kbc_geq<i>(rho, rhom1, ux, uy, uz, u2);
        const float ds = (4.5f * wgt(i)) * kbc_cdc<i>(dxx, dyy, dzz, pxy, pxz, pyz);
        const float dh = kbc_dh(I, geq, ds);
        const float r = dh / (geq + wgt(i));
        sh = sh + ds * r;
        hh = hh + dh * r;
    });
    const float beta = 0.5f * w;
    const float ib = 1.0f / beta;
    const float gamma =
        fminf(fmaxf(hh > 0.0f ? ib - (2.0f - ib) * sh / hh : 2.0f, 0.0f), 2.0f * ib);
    float a = 0.0f, uF = 0.0f;
    if constexpr (FORCE) {
        a = 1.0f - 0.5f * w;
        uF = ux * Fx + uy * Fy + uz * Fz;
    }
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const float geq = kbc_geq<i>(rho, rhom1, ux, uy, uz, u2);
        const float ds = (4.5f * wgt(i)) * kbc_cdc<i>(dxx, dyy, dzz, pxy, pxz, pyz);
        const float dh = kbc_dh(I, geq, ds);
        float v;
        if constexpr (FORCE) {
            const float cF = i == 0 ? 0.0f : cdot<i>(Fx, Fy, Fz);
            const float cu = i == 0 ? 0.0f : cdot<i>(ux, uy, uz);
            const float dk = (-1.5f * wgt(i)) * cF;
            v = fh[i] - beta * (2.0f * (ds + dk) + gamma * dh);
            v = v + a * wgt(i) * (3.0f * cF + 9.0f * cu * cF - 3.0f * uF);
        } else {
            v = fh[i] - beta * (2.0f * ds + gamma * dh);
        }
        fh[i] = v;
    });
}

// Collision, Kernels.metal:105-228. FEAT 3 is the KBC collision (sponge and
// force as FEAT 1; no LES, no Noble-Torczynski cells).
template <int FEAT, int ARITH = ARITH_REFERENCE>
__device__ __forceinline__ void collide(float (&fh)[19], const StepArgs& a, int x, float eps,
                                        float Fx, float Fy, float Fz, float& ntx, float& nty,
                                        float& ntz) {
    float wp = a.omega, wm = a.omega_minus;
    if constexpr (FEAT) {
        if ((float)x > a.sponge_x0) {  // viscous sponge, Kernels.metal:112-123
            const float frac = fminf(((float)x - a.sponge_x0) * a.sponge_inv_w, 1.0f);
            const float tau0 = 1.0f / wp;
            const float tauS = tau0 + frac * (a.sponge_tau - tau0);
            if (a.omega_minus == a.omega) {
                wp = 1.0f / tauS;
                wm = wp;
            } else {
                const float lambda = (1.0f / wp - 0.5f) * (1.0f / wm - 0.5f);
                wp = 1.0f / tauS;
                wm = 1.0f / (0.5f + lambda / (tauS - 0.5f));
            }
        }
    }
    float rhom1 = fh[0];
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
    const float rho = 1.0f + rhom1;
    const float inv = 1.0f / rho;
    float ux, uy, uz;
    if constexpr (FEAT) {
        if constexpr (ARITH == ARITH_REFERENCE) {
            ux = (px + 0.5f * Fx) * inv;
            uy = (py + 0.5f * Fy) * inv;
            uz = (pz + 0.5f * Fz) * inv;
        } else {
            ux = fmaf(0.5f, Fx, px) * inv;
            uy = fmaf(0.5f, Fy, py) * inv;
            uz = fmaf(0.5f, Fz, pz) * inv;
        }
    } else {
        ux = px * inv;
        uy = py * inv;
        uz = pz * inv;
    }
    if constexpr (FEAT == 3) {  // KBC (the arithmetic only changes u); no LES, no NT cells
        const float u2k = ux * ux + uy * uy + uz * uz;
        // the Guo source where the cell's force is nonzero
        if (a.force_on && (Fx != 0.0f || Fy != 0.0f || Fz != 0.0f))
            relax_kbc<true>(fh, wp, rho, rhom1, ux, uy, uz, u2k, Fx, Fy, Fz);
        else relax_kbc<false>(fh, wp, rho, rhom1, ux, uy, uz, u2k, Fx, Fy, Fz);
        return;
    }
    const float u2 = ARITH == ARITH_REFERENCE ? ux * ux + uy * uy + uz * uz
                                              : fmaf(uz, uz, fmaf(uy, uy, ux * ux));

    if constexpr (FEAT == 2) {
        if (a.c_smago > 0.0f) {  // Smagorinsky LES, Kernels.metal:140-167
            float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
            // second moments of d_i: d = f - feq (reference), or the raw f (fused)
            auto second_moments = [&](auto dof) {
                sfor<1, 19>([&](auto I) {
                    constexpr int i = I;
                    const float d = dof(I);
                    // first nonzero term of each sum starts it (index 1, 3, 5, 7, 11, 15)
                    if constexpr (dcx(i) != 0) pxx = (i == 1) ? d : pxx + d;
                    if constexpr (dcy(i) != 0) pyy = (i == 3) ? d : pyy + d;
                    if constexpr (dcz(i) != 0) pzz = (i == 5) ? d : pzz + d;
                    if constexpr (dcx(i) * dcy(i) > 0) pxy = (i == 7) ? d : pxy + d;
                    if constexpr (dcx(i) * dcy(i) < 0) pxy -= d;
                    if constexpr (dcx(i) * dcz(i) > 0) pxz = (i == 11) ? d : pxz + d;
                    if constexpr (dcx(i) * dcz(i) < 0) pxz -= d;
                    if constexpr (dcy(i) * dcz(i) > 0) pyz = (i == 15) ? d : pyz + d;
                    if constexpr (dcy(i) * dcz(i) < 0) pyz -= d;
                });
            };
            float Q, tauEff;
            // 1 / wp; outside the sponge wp is omega and its reciprocal comes
            // with the launch (the same FP32 division, done once on the host)
            const float tau0 = wp == a.omega ? a.tau0 : 1.0f / wp;
            if constexpr (ARITH == ARITH_REFERENCE) {
                second_moments([&](auto I) {
                    constexpr int i = I;
                    constexpr float w = wgt(i);
                    const float cu = 3.0f * cdot<i>(ux, uy, uz);
                    const float feq = w * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
                    return fh[i] - feq;
                });
                Q = sqrtf(pxx * pxx + pyy * pyy + pzz * pzz +
                          2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
                tauEff = 0.5f * (tau0 + sqrtf(tau0 * tau0 + 25.455844f * a.c_smago * Q * inv));
            } else {
                // The equilibrium's second moments are known in closed form,
                // sum_i c_ia c_ib feq_i = rhom1/3 delta_ab + rho u_a u_b (shifted
                // DDFs), so Pi_neq = sum_i c_ia c_ib f_i minus them: no per-direction
                // equilibria.
                second_moments([&](auto I) { return fh[I]; });
                const float r3 = rhom1 * (1.0f / 3.0f);
                const float rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
                pxx = fmaf(-rux, ux, pxx - r3);
                pyy = fmaf(-ruy, uy, pyy - r3);
                pzz = fmaf(-ruz, uz, pzz - r3);
                pxy = fmaf(-rux, uy, pxy);
                pxz = fmaf(-rux, uz, pxz);
                pyz = fmaf(-ruy, uz, pyz);
                Q = sqrtf(fmaf(pzz, pzz, fmaf(pyy, pyy, pxx * pxx)) +
                          2.0f * fmaf(pyz, pyz, fmaf(pxz, pxz, pxy * pxy)));
                tauEff = 0.5f * (tau0 + sqrtf(fmaf(tau0, tau0, 25.455844f * a.c_smago * Q * inv)));
            }
            if (a.omega_minus == a.omega) {
                wp = 1.0f / tauEff;
                wm = wp;
            } else {
                const float lambda = (1.0f / wp - 0.5f) * (1.0f / wm - 0.5f);
                wp = 1.0f / tauEff;
                wm = 1.0f / (0.5f + lambda / (tauEff - 0.5f));
            }
        }
    }
    auto relax_any = [&](auto force, auto nt) {
        constexpr bool FO = decltype(force)::value, NO = decltype(nt)::value;
        if constexpr (ARITH == ARITH_REFERENCE)
            relax<FO, NO>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty, ntz);
        else
            relax_fused<FO, NO>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty,
                                ntz);
    };
    using T = std::true_type;
    using F = std::false_type;
    if constexpr (FEAT) {
        if (eps == 0.0f) {
            if (a.force_on) relax_any(T{}, F{});
            else relax_any(F{}, F{});
        } else {
            if (a.force_on) relax_any(T{}, T{});
            else relax_any(F{}, T{});
        }
    } else {
        Fx = Fy = Fz = 0.0f;
        relax_any(F{}, F{});
    }
}

template <int FEAT>
__device__ __forceinline__ void cell_force(const StepArgs& a, uint32_t n, float& Fx, float& Fy,
                                           float& Fz) {
    Fx = a.fx; Fy = a.fy; Fz = a.fz;
    if constexpr (FEAT) {
        if (a.ffield != nullptr) {
            Fx = a.fx + a.ffield[n];
            Fy = a.fy + a.ffield[a.ffield_plane + n];
            Fz = a.fz + a.ffield[2u * a.ffield_plane + n];
        }
    }
}

// c_i * v added to (ax, ay, az), zero components skipped.
template <int I>
__device__ __forceinline__ void acc_add(float& ax, float& ay, float& az, float v) {
    if constexpr (dcx(I) > 0) ax += v;
    if constexpr (dcx(I) < 0) ax -= v;
    if constexpr (dcy(I) > 0) ay += v;
    if constexpr (dcy(I) < 0) ay -= v;
    if constexpr (dcz(I) > 0) az += v;
    if constexpr (dcz(I) < 0) az -= v;
}
template <int I>
__device__ __forceinline__ void acc_sub(float& ax, float& ay, float& az, float v) {
    if constexpr (dcx(I) > 0) ax -= v;
    if constexpr (dcx(I) < 0) ax += v;
    if constexpr (dcy(I) > 0) ay -= v;
    if constexpr (dcy(I) < 0) ay += v;
    if constexpr (dcz(I) > 0) az -= v;
    if constexpr (dcz(I) < 0) az += v;
}

// Wrapped neighbour offsets of one cell: the linear offset of x-1, x+1, ...
struct NbrOffsets {
    int xm, xp, ym, yp, zm, zp;
    __device__ __forceinline__ NbrOffsets(int x, int y, int z, int nx, int ny, int nz) {
        const int nxy = nx * ny;
        xm = (x == 0) ? nx - 1 : -1;
        xp = (x == nx - 1) ? -(nx - 1) : 1;
        ym = (y == 0) ? (ny - 1) * nx : -nx;
        yp = (y == ny - 1) ? -(ny - 1) * nx : nx;
        zm = (z == 0) ? (nz - 1) * nxy : -nxy;
        zp = (z == nz - 1) ? -(nz - 1) * nxy : nxy;
    }
    template <int DX, int DY, int DZ>
    __device__ __forceinline__ int off() const {
        return (DX > 0 ? xp : (DX < 0 ? xm : 0)) + (DY > 0 ? yp : (DY < 0 ? ym : 0)) +
               (DZ > 0 ? zp : (DZ < 0 ? zm : 0));
    }
};

// Deferred moving-wall corrections of the gathered DDFs, Kernels.metal:292-314.
// Bit i of `abb` is set for each link reflected from an outflow wall.
template <bool PROBE>
__device__ __forceinline__ void moving_wall_loads(float (&fh)[19], const StepArgs& a,
                                                  const WallVel& wv, uint32_t wb, uint32_t lm,
                                                  int x, int y, int z, float& ax, float& ay,
                                                  float& az, uint32_t& abb) {
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int bit = opp(i) - 1;
        if (((wb >> bit) & 1u) && ((lm >> bit) & 1u)) {
            const int sy = wrapi(y - dcy(i), a.ny);
            const uint32_t s = (uint32_t(wrapi(z - dcz(i), a.nz)) * uint32_t(a.ny) + uint32_t(sy)) *
                                   uint32_t(a.nx) +
                               uint32_t(wrapi(x - dcx(i), a.nx));
            const uint8_t wf = a.cell[s] & CELL_TYPE_MASK;
            if (wf == CELL_OUTFLOW) {
                fh[i] = -fh[i];
                abb |= 1u << i;
            } else {
                float uwx, uwy, uwz;
                wall_velocity(wf, sy, a, wv, uwx, uwy, uwz);
                const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                fh[i] += corr;
                if constexpr (PROBE) acc_sub<i>(ax, ay, az, corr);
            }
        }
    });
}

// Pressure outflow (anti-bounce-back at rho_w = 1 with its velocity terms):
// the reflected shifted DDF of link i gains w_i (9 (c_i . u)^2 - 3 u^2), the
// equilibrium part 2 w_i rho_w (1 + 4.5 (c_i . u)^2 - 1.5 u^2) of raw DDFs
// minus the 2 w_i of the shift. u = p / rho of the wall cell's DDFs, no
// force term: the gathered ones (reflections without the terms) for the
// incoming links, the post-collision ones for the outgoing links.
struct OutflowVel {
    float ux = 0.f, uy = 0.f, uz = 0.f, u2 = 0.f;
    __device__ __forceinline__ void estimate(const float (&fh)[19]) {
        float rhom1 = fh[0];
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
        const float inv = 1.0f / (1.0f + rhom1);
        ux = px * inv;
        uy = py * inv;
        uz = pz * inv;
        u2 = ux * ux + uy * uy + uz * uz;
    }
    template <int I>
    __device__ __forceinline__ float term() const {
        const float cu = cdot<I>(ux, uy, uz);
        return wgt(I) * (9.0f * cu * cu - 3.0f * u2);
    }
};

// Scatter with moving-wall corrections, Kernels.metal:317-350.
template <typename S, bool PROBE>
__device__ __forceinline__ void moving_wall_stores(S* __restrict__ f, const float (&fh)[19],
                                                   const StepArgs& a, const WallVel& wv,
                                                   uint32_t n, uint32_t wb, uint32_t lm, int x,
                                                   int y, int z, const NbrOffsets& nb, float& ax,
                                                   float& ay, float& az, const OutflowVel& ov) {
    const uint64_t P = a.plane;
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        if (!((wb >> (i - 1)) & 1u)) {
            store_ddf<S>(f + uint64_t(i) * P + uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>()), fh[i]);
        } else {
            float sv = fh[i];
            float out = sv;
            if ((lm >> (i - 1)) & 1u) {
                const int dy = wrapi(y + dcy(i), a.ny);
                const uint32_t d = (uint32_t(wrapi(z + dcz(i), a.nz)) * uint32_t(a.ny) + uint32_t(dy)) *
                                       uint32_t(a.nx) +
                                   uint32_t(wrapi(x + dcx(i), a.nx));
                const uint8_t wf = a.cell[d] & CELL_TYPE_MASK;
                if (wf == CELL_OUTFLOW) {
                    sv = -fh[i];
                    out = a.outflow_pressure ? sv + ov.template term<i>() : sv;
                } else {
                    float uwx, uwy, uwz;
                    wall_velocity(wf, dy, a, wv, uwx, uwy, uwz);
                    const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                    out = sv - corr;
                }
            }
            store_ddf<S>(f + uint64_t(opp(i)) * P + n, out);
            if constexpr (PROBE) acc_add<i>(ax, ay, az, sv + 2.0f * wgt(i));
        }
    });
}


// |u|^2 of a cell's natural-slot DDFs, formed as momentsEven does
// (Kernels.metal:368-379: division by rho) and as the host energy loop squares
// it (Cases.swift:1242).
__device__ __forceinline__ float cell_u2(const float (&fh)[19], float Fx, float Fy, float Fz) {
    float rhom1 = fh[0];
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
    const float rho = 1.0f + rhom1;
    const float ux = (px + 0.5f * Fx) / rho, uy = (py + 0.5f * Fy) / rho,
                uz = (pz + 0.5f * Fz) / rho;
    return ux * ux + uy * uy + uz * uz;
}

// Register pressure fence: the pointer passes through an empty asm
// statement, so addresses formed from it afterwards are computed afresh
// instead of being kept alive from the loads. In both AA passes the stores go
// to the very slots the loads came from, and keeping those 19 addresses (two
// registers each) across the collision would cost more registers than
// recomputing them costs instructions.
template <typename P>
__device__ __forceinline__ void forget_ptr(P& p) {
    asm volatile("" : "+l"(p));
}

// Even (in-cell) pass of one cell, Kernels.metal:252-260. Non-fluid cells are
// skipped. With LOG, u2 receives |u|^2 of the state before the step.
// OUT: honour StepArgs::f_out (out-of-place pass); on by default where the
// lattice has walls, and for the block-list kernels of the bulk / boundary split.
// GEO 2 (blocks of the x-face list, see odd_cell_xface): the non-fluid cells
// are the columns x = 0 and x = nx - 1 and no cell is partially saturated, so
// no cell byte is read.
// PO: address the planes through the launch's 32-bit plane offsets
// (StepArgs::poff, valid when 19 planes fit 2^32 elements) from a per-thread
// base pointer: one wide multiply-add per address instead of a 64-bit add of
// plane * i. Used by the wall-free and x-face block-list kernels.
template <typename S, int GEO, int FEAT, bool LOG = false, bool CG = false,
          int ARITH = ARITH_REFERENCE, bool OUT = (GEO != 0), bool PO = false>
__device__ __forceinline__ void even_cell(const StepArgs& a, int x, int y, int z,
                                          float* u2 = nullptr) {
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    float eps = 0.0f;
    if constexpr (GEO == 2) {
        if (x == 0 || x == a.nx - 1) return;
    }
    if constexpr (GEO == 1) {
        const uint8_t c = a.cell[n];
        if (c & CELL_TYPE_MASK) return;
        if constexpr (FEAT) {
            if (c & CELL_EPS_BIT) eps = a.eps[n];
        }
    }
    S* __restrict__ f = static_cast<S*>(a.f);
    const uint64_t P = a.plane;
    float fh[19];
    if constexpr (PO) {
        const S* fb = f + n;
        sfor<0, 19>([&](auto I) { fh[I] = load_slot<S, CG>(fb + a.poff[I]); });
    } else {
        sfor<0, 19>([&](auto I) { fh[I] = load_slot<S, CG>(f + uint64_t(I) * P + n); });
    }
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    if constexpr (LOG) *u2 = cell_u2(fh, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT, ARITH>(fh, a, x, eps, Fx, Fy, Fz, ntx, nty, ntz);
    forget_ptr(f);
    if constexpr (OUT) {  // out of place
        if (a.f_out != nullptr) f = static_cast<S*>(a.f_out);
    }
    if constexpr (PO) {
        S* fb = f + n;
        store_ddf<S>(fb, fh[0]);
        sfor<1, 19>([&](auto I) { store_ddf<S>(fb + a.poff[opp(I)], fh[I]); });
    } else {
        store_ddf<S>(f + n, fh[0]);
        sfor<1, 19>([&](auto I) { store_ddf<S>(f + uint64_t(opp(I)) * P + n, fh[I]); });
    }
}

// Odd (streaming) pass of one cell with halfway / moving-wall bounce-back,
// Kernels.metal:261-354. With PROBE the cell's momentum-exchange force is
// returned in contrib when the cell is a boundary cell inside the probe box.
template <typename S, int GEO, int FEAT, bool PROBE, bool CG = false,
          int ARITH = ARITH_REFERENCE, bool OUT = (GEO != 0), bool PO = false>
__device__ __forceinline__ void odd_cell(const StepArgs& a, const WallVel& wv, int x, int y,
                                         int z, double (&contrib)[3]) {
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    uint32_t g = 0;
    if constexpr (GEO) {
        g = a.geo[n];
        if (g & GEO_NONFLUID) return;
    }
    S* __restrict__ f = static_cast<S*>(a.f);
    const uint64_t P = a.plane;
    const NbrOffsets nb(x, y, z, a.nx, a.ny, a.nz);
    const uint32_t wb = g & GEO_WALL_BITS;
    float eps = 0.0f;
    if constexpr (GEO && FEAT) {
        if (g & GEO_EPS) eps = a.eps[n];
    }
    float ax = 0.f, ay = 0.f, az = 0.f;
    float fh[19];
    fh[0] = load_slot<S, CG>(f + n);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        const uint32_t src = uint32_t(int(n) + nb.template off<-dcx(i), -dcy(i), -dcz(i)>());
        if constexpr (GEO) {
            const bool bb = (wb >> (o - 1)) & 1u;
            const uint64_t idx = bb ? (uint64_t(i) * P + n) : (uint64_t(o) * P + src);
            fh[i] = load_slot<S, CG>(f + idx);
            if constexpr (PROBE) {
                if (bb) acc_sub<i>(ax, ay, az, fh[i]);
            }
        } else {
            if constexpr (PO) fh[i] = load_slot<S, CG>(f + (a.poff[o] + src));
            else fh[i] = load_slot<S, CG>(f + uint64_t(o) * P + src);
        }
    });
    uint32_t lm = 0;
    if constexpr (GEO) {
        if (g & GEO_MOVING) {
            lm = a.lmask[n];
            uint32_t abb = 0;
            moving_wall_loads<PROBE>(fh, a, wv, wb, lm, x, y, z, ax, ay, az, abb);
            if (a.outflow_pressure) {
                OutflowVel ov;
                ov.estimate(fh);
                sfor<1, 19>([&](auto I) {
                    if ((abb >> int(I)) & 1u) fh[I] += ov.template term<I>();
                });
            }
        }
    }
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT, ARITH>(fh, a, x, eps, Fx, Fy, Fz, ntx, nty, ntz);
    if constexpr (PROBE) {
        ax += ntx;
        ay += nty;
        az += ntz;
    }
    forget_ptr(f);
    if constexpr (OUT) {  // out of place
        if (a.f_out != nullptr) f = static_cast<S*>(a.f_out);
    }
    store_ddf<S>(f + n, fh[0]);
    if constexpr (GEO) {
        // A warp that holds a moving-wall cell runs the moving-wall scatter for
        // all its lanes (it covers plain and bounce-back links too) instead of
        // running both scatters one after the other; the stored values are the same.
        if (!__any_sync(__activemask(), (g & GEO_MOVING) != 0u)) {
            sfor<1, 19>([&](auto I) {
                constexpr int i = I;
                constexpr int o = opp(i);
                const bool bb = (wb >> (i - 1)) & 1u;
                const uint32_t dst = uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>());
                const uint64_t idx = bb ? (uint64_t(o) * P + n) : (uint64_t(i) * P + dst);
                store_ddf<S>(f + idx, fh[i]);
                if constexpr (PROBE) {
                    if (bb) acc_add<i>(ax, ay, az, fh[i] + 2.0f * wgt(i));
                }
            });
        } else {
            OutflowVel ov;
            if (a.outflow_pressure && (g & GEO_MOVING)) ov.estimate(fh);
            moving_wall_stores<S, PROBE>(f, fh, a, wv, n, wb, lm, x, y, z, nb, ax, ay, az, ov);
        }
    } else {
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            const uint32_t dst = uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>());
            if constexpr (PO) store_ddf<S>(f + (a.poff[i] + dst), fh[i]);
            else store_ddf<S>(f + uint64_t(i) * P + dst, fh[i]);
        });
    }
    if constexpr (PROBE) {
        if ((wb != 0u || eps > 0.0f) && x >= a.box_x0 && x <= a.box_x1 && y >= a.box_y0 &&
            y <= a.box_y1) {
            contrib[0] = (double)ax;
            contrib[1] = (double)ay;
            contrib[2] = (double)az;
        }
    }
}

// Odd pass of one cell of an x-face block: a block whose only walls are
// velocity-inflow columns at x = 0 and x = nx - 1, every link of a cell at
// x = 1 (x = nx - 2) toward x = 0 (x = nx - 1) a moving-wall link and no other
// link a wall link, and no cell partially saturated (the host checks this cell
// by cell before it lists the block). The wall links then follow from x alone:
// no geometry word, moving-link mask or wall cell byte is read. The values are
// the ones odd_cell computes for these cells (the same gather, moving-wall
// corrections of Kernels.metal:292-314 and 317-350, collision and scatter);
// inflow walls take no outflow terms.
template <typename S, int FEAT, int ARITH = ARITH_REFERENCE, bool PO = false>
__device__ __forceinline__ void odd_cell_xface(const StepArgs& a, const WallVel& wv, int x, int y,
                                               int z) {
    if (x == 0 || x == a.nx - 1) return;
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    const bool wl = x == 1, wr = x == a.nx - 2;  // next to the x = 0 / x = nx - 1 wall
    S* __restrict__ f = static_cast<S*>(a.f);
    const uint64_t P = a.plane;
    const NbrOffsets nb(x, y, z, a.nx, a.ny, a.nz);
    float fh[19];
    fh[0] = load_slot<S, false>(f + n);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        const uint32_t src = uint32_t(int(n) + nb.template off<-dcx(i), -dcy(i), -dcz(i)>());
        if constexpr (dcx(i) == 0) {
            if constexpr (PO) fh[i] = load_slot<S, false>(f + (a.poff[o] + src));
            else fh[i] = load_slot<S, false>(f + uint64_t(o) * P + src);
        } else {
            // n - c_i lies in a wall column: the link reflects within the cell
            const bool bb = dcx(i) > 0 ? wl : wr;
            if constexpr (PO)
                fh[i] = load_slot<S, false>(f + (bb ? a.poff[i] + n : a.poff[o] + src));
            else
                fh[i] = load_slot<S, false>(f + (bb ? uint64_t(i) * P + n : uint64_t(o) * P + src));
        }
    });
    if (wl || wr) {
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            if constexpr (dcx(i) != 0) {
                if (dcx(i) > 0 ? wl : wr) {
                    float uwx, uwy, uwz;
                    wall_velocity(CELL_INFLOW, wrapi(y - dcy(i), a.ny), a, wv, uwx, uwy, uwz);
                    const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                    fh[i] += corr;
                }
            }
        });
    }
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT, ARITH>(fh, a, x, 0.0f, Fx, Fy, Fz, ntx, nty, ntz);
    forget_ptr(f);
    if (a.f_out != nullptr) f = static_cast<S*>(a.f_out);
    store_ddf<S>(f + n, fh[0]);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        const uint32_t dst = uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>());
        if constexpr (dcx(i) == 0) {
            if constexpr (PO) store_ddf<S>(f + (a.poff[i] + dst), fh[i]);
            else store_ddf<S>(f + uint64_t(i) * P + dst, fh[i]);
        } else {
            // n + c_i lies in a wall column: store into the cell's own opposite slot
            const bool bb = dcx(i) < 0 ? wl : wr;
            float out = fh[i];
            if (bb) {
                float uwx, uwy, uwz;
                wall_velocity(CELL_INFLOW, wrapi(y + dcy(i), a.ny), a, wv, uwx, uwy, uwz);
                const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                out = fh[i] - corr;
            }
            if constexpr (PO)
                store_ddf<S>(f + (bb ? a.poff[opp(i)] + n : a.poff[i] + dst), out);
            else
                store_ddf<S>(f + (bb ? uint64_t(opp(i)) * P + n : uint64_t(i) * P + dst), out);
        }
    });
}

}  // namespace stro
