// Discrete adjoint of the D3Q19 AA step (reverse mode, FP32).
//
// Objective: J = sum over the odd steps t of w_t * dir . F_box(t), with F_box
// the momentum-exchange force of the odd pass summed over the probe box (the
// reference's force probe, Kernels.metal:263-353) and w_t = 1/K for the K odd
// steps of the window (time-averaged drag when dir = x).
//
// One forward step maps the slots a cell reads (set R_n) to the slots it
// writes (set W_n) through the per-cell collision; in the AA pattern
// R_n = W_n, so the adjoint step is again an in-place pass over the adjoint
// array lam: each cell reads lam at the slots it wrote, applies the transposed
// Jacobian of its local update, and writes lam at the slots it read. The
// Jacobian is applied by a hand-written reverse pass of collide() (TRT + Guo
// force + Smagorinsky + Noble-Torczynski; the sponge only changes constants),
// which recomputes the forward intermediates from the stored input state.
// Bounce-back and moving-wall terms are permutations, signs and constants.
//
// Gradients are accumulated per cell: dJ/d eps for Noble-Torczynski cells
// (eps != 0; a cell with eps = 0 takes the plain path, which does not depend
// on eps) and dJ/dF for the per-cell Guo force field. No atomics: every cell
// is owned by one thread per pass.
#include "lbm_adjoint.h"
#include "lbm_cell.cuh"

namespace stro {

namespace {

// c_i . (bx, by, bz) for the compile-time direction I (zero components skipped)
template <int I>
__device__ __forceinline__ float cdotv(float bx, float by, float bz) {
    return cdot<I>(bx, by, bz);
}

template <int I>
__device__ __forceinline__ void add_c(float& ox, float& oy, float& oz, float v) {
    if constexpr (dcx(I) > 0) ox += v;
    if constexpr (dcx(I) < 0) ox -= v;
    if constexpr (dcy(I) > 0) oy += v;
    if constexpr (dcy(I) < 0) oy -= v;
    if constexpr (dcz(I) > 0) oz += v;
    if constexpr (dcz(I) < 0) oz -= v;
}

// Reverse of collide() for one cell.
//   fh      : pre-collision populations (after gather and wall corrections)
//   ab      : in  dJ/d(post-collision population i); out dJ/d(fh_i)
//   ntb     : dJ/d(Noble-Torczynski force of the cell)
//   force_terms: differentiate the Guo source terms (needed for dJ/dF even at F = 0)
// LES / NT: whether the lattice can have a Smagorinsky model / Noble-Torczynski
// cells at all; a pass without them compiles their blocks out (fewer
// registers), with the same values for the cells it runs.
template <bool LES, bool NT>
__device__ __forceinline__ void collide_adj(const float (&fh)[19], const StepArgs& a, int x,
                                            float eps, float Fx, float Fy, float Fz,
                                            float (&ab)[19], float ntbx, float ntby, float ntbz,
                                            bool force_terms, float& epsb, float& Fbx,
                                            float& Fby, float& Fbz) {
    // ---------------- forward recompute
    float wp = a.omega, wm = a.omega_minus;
    if ((float)x > a.sponge_x0) {
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
    const float wp0 = wp, wm0 = wm;
    float rhom1 = fh[0];
    sfor<1, 19>([&](auto I) { rhom1 += fh[I]; });
    const float rho = 1.0f + rhom1;
    const float inv = 1.0f / rho;
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
    const float qx = px + 0.5f * Fx, qy = py + 0.5f * Fy, qz = pz + 0.5f * Fz;
    const float ux = qx * inv, uy = qy * inv, uz = qz * inv;
    const float u2 = ux * ux + uy * uy + uz * uz;
    const bool les = LES && a.c_smago > 0.0f;
    const bool srt = a.omega_minus == a.omega;
    float Q = 0.f, S = 0.f, te = 0.f, lam = 0.f;
    float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
    const float Kc = 25.455844f * a.c_smago;
    if (les) {
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            constexpr float w = wgt(i);
            const float cu = 3.0f * cdot<i>(ux, uy, uz);
            const float d = fh[i] - w * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
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
        Q = sqrtf(pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
        const float tau0 = 1.0f / wp0;
        S = sqrtf(tau0 * tau0 + Kc * Q * inv);
        te = 0.5f * (tau0 + S);
        wp = 1.0f / te;
        if (srt) {
            wm = wp;
        } else {
            lam = (1.0f / wp0 - 0.5f) * (1.0f / wm0 - 0.5f);
            wm = 1.0f / (0.5f + lam / (te - 0.5f));
        }
    }
    const float uF = ux * Fx + uy * Fy + uz * Fz;
    const float ap = 1.0f - 0.5f * wp;
    const float am = 1.0f - 0.5f * wm;
    const float W0 = wgt(0);
    const float feq0 = W0 * (rhom1 - 1.5f * rho * u2);
    const float s0 = force_terms ? W0 * ap * (-3.0f * uF) : 0.0f;
    const bool nt = NT && eps != 0.0f;
    const float tw = 1.0f / wp - 0.5f;
    const float Dn = (1.0f - eps) + tw;
    const float B = nt ? eps * tw / Dn : 0.0f;
    const float omb = 1.0f - B;

    // ---------------- reverse
    float rhom1b = 0.f, rhob = 0.f, invb = 0.f, uxb = 0.f, uyb = 0.f, uzb = 0.f, u2b = 0.f;
    float wpb = 0.f, wmb = 0.f, apb = 0.f, amb = 0.f, uFb = 0.f, Bb = 0.f, ombb = 0.f;
    Fbx = Fby = Fbz = 0.f;
    epsb = 0.f;
    {  // rest direction: fh0' = fh0 + omb * (wp (feq0 - fh0) + s0)
        const float X = wp * (feq0 - fh[0]) + s0;
        const float a0 = ab[0];
        float fb0 = a0;
        ombb += X * a0;
        const float Xb = omb * a0;
        wpb += (feq0 - fh[0]) * Xb;
        const float feq0b = wp * Xb;
        fb0 -= wp * Xb;
        rhom1b += W0 * feq0b;
        rhob += -1.5f * W0 * u2 * feq0b;
        u2b += -1.5f * W0 * rho * feq0b;
        if (force_terms) {
            apb += -3.0f * W0 * uF * Xb;
            uFb += -3.0f * W0 * ap * Xb;
        }
        ab[0] = fb0;
    }
    sfor<0, 9>([&](auto P) {
        constexpr int i = 2 * P + 1;
        constexpr int j = i + 1;
        constexpr float w = wgt(i);
        const float fi = fh[i], fj = fh[j];
        const float cu = 3.0f * cdot<i>(ux, uy, uz);
        const float feqp = w * (rhom1 + rho * (0.5f * cu * cu - 1.5f * u2));
        const float feqm = w * rho * cu;
        const float fp = 0.5f * (fi + fj);
        const float fm = 0.5f * (fi - fj);
        const float dp = wp * (feqp - fp);
        const float dm = wm * (feqm - fm);
        float cF = 0.f, sm = 0.f, sp = 0.f;
        if (force_terms) {
            cF = cdot<i>(Fx, Fy, Fz);
            sm = w * am * (3.0f * cF);
            sp = w * ap * (3.0f * cu * cF - 3.0f * uF);
        }
        const float up = dp + dm + sp + sm;
        const float um = dp - dm + sp - sm;
        const float ai = ab[i], aj = ab[j];
        float fbi = ai, fbj = aj;
        const float upb = omb * ai, umb = omb * aj;
        ombb += up * ai + um * aj;
        if (nt) {
            const float t = 2.0f * cdotv<i>(ntbx, ntby, ntbz);
            const float bb = ai - aj - t;
            Bb += (fj - fi) * bb;
            if (B == 1.0f) {
                // Fully covered cell (eps = 1, so B = 1 exactly and 1 - B = 0):
                // the update is a pure exchange of f_i and f_j, and so is its
                // reverse. Written out, not as ai - B * bb: inside a solid body
                // the adjoint is only exchanged, never damped, and grows over
                // the window; the general form then cancels the large value
                // against itself and loses the solid-fraction gradient's
                // digits (1% off the FP64 adjoint after 2,000 steps of the C3
                // cylinder; this form agrees to 3e-5, as FP64 does).
                fbi = aj + t;
                fbj = ai - t;
            } else {
                fbj += B * bb;
                fbi -= B * bb;
            }
        }
        const float dpb = upb + umb, dmb = upb - umb;
        wpb += (feqp - fp) * dpb;
        const float feqpb = wp * dpb, fpb = -wp * dpb;
        wmb += (feqm - fm) * dmb;
        const float feqmb = wm * dmb, fmb = -wm * dmb;
        fbi += 0.5f * (fpb + fmb);
        fbj += 0.5f * (fpb - fmb);
        rhom1b += w * feqpb;
        rhob += w * (0.5f * cu * cu - 1.5f * u2) * feqpb + w * cu * feqmb;
        float cub = w * rho * cu * feqpb + w * rho * feqmb;
        u2b += -1.5f * w * rho * feqpb;
        if (force_terms) {
            const float spb = upb + umb, smb = upb - umb;
            amb += 3.0f * w * cF * smb;
            const float cFb = 3.0f * w * am * smb + 3.0f * w * ap * cu * spb;
            apb += w * (3.0f * cu * cF - 3.0f * uF) * spb;
            cub += 3.0f * w * ap * cF * spb;
            uFb += -3.0f * w * ap * spb;
            add_c<i>(Fbx, Fby, Fbz, cFb);
        }
        add_c<i>(uxb, uyb, uzb, 3.0f * cub);
        ab[i] = fbi;
        ab[j] = fbj;
    });
    Bb += -ombb;
    if (nt) {
        const float D2 = Dn * Dn;
        epsb = Bb * tw * (1.0f + tw) / D2;
        const float twb = Bb * eps * (1.0f - eps) / D2;
        wpb += -twb / (wp * wp);
    }
    wpb += -0.5f * apb;
    wmb += -0.5f * amb;
    if (force_terms) {
        uxb += Fx * uFb;
        uyb += Fy * uFb;
        uzb += Fz * uFb;
        Fbx += ux * uFb;
        Fby += uy * uFb;
        Fbz += uz * uFb;
    }
    if (les) {
        float teb;
        if (srt) {
            wpb += wmb;
            teb = -wp * wp * wpb;
        } else {
            const float g = 0.5f + lam / (te - 0.5f);
            const float tm = te - 0.5f;
            teb = -wp * wp * wpb + wmb * lam / (g * g * tm * tm);
        }
        const float Qb = teb * Kc * inv / (4.0f * S);
        invb += teb * Kc * Q / (4.0f * S);
        float pxxb = 0.f, pyyb = 0.f, pzzb = 0.f, pxyb = 0.f, pxzb = 0.f, pyzb = 0.f;
        if (Q > 0.0f) {
            const float r = Qb / Q;
            pxxb = pxx * r;
            pyyb = pyy * r;
            pzzb = pzz * r;
            pxyb = 2.0f * pxy * r;
            pxzb = 2.0f * pxz * r;
            pyzb = 2.0f * pyz * r;
        }
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            constexpr float w = wgt(i);
            float db = 0.f;
            if constexpr (dcx(i) != 0) db += pxxb;
            if constexpr (dcy(i) != 0) db += pyyb;
            if constexpr (dcz(i) != 0) db += pzzb;
            if constexpr (dcx(i) * dcy(i) > 0) db += pxyb;
            if constexpr (dcx(i) * dcy(i) < 0) db -= pxyb;
            if constexpr (dcx(i) * dcz(i) > 0) db += pxzb;
            if constexpr (dcx(i) * dcz(i) < 0) db -= pxzb;
            if constexpr (dcy(i) * dcz(i) > 0) db += pyzb;
            if constexpr (dcy(i) * dcz(i) < 0) db -= pyzb;
            ab[i] += db;
            const float feqb = -db;
            const float cu = 3.0f * cdot<i>(ux, uy, uz);
            rhom1b += w * feqb;
            rhob += w * (cu + 0.5f * cu * cu - 1.5f * u2) * feqb;
            u2b += -1.5f * w * rho * feqb;
            add_c<i>(uxb, uyb, uzb, 3.0f * w * rho * (1.0f + cu) * feqb);
        });
    }
    uxb += 2.0f * ux * u2b;
    uyb += 2.0f * uy * u2b;
    uzb += 2.0f * uz * u2b;
    const float pxb = inv * uxb, pyb = inv * uyb, pzb = inv * uzb;
    Fbx += 0.5f * inv * uxb;
    Fby += 0.5f * inv * uyb;
    Fbz += 0.5f * inv * uzb;
    invb += qx * uxb + qy * uyb + qz * uzb;
    rhob += -inv * inv * invb;
    rhom1b += rhob;
    ab[0] += rhom1b;
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        ab[i] += rhom1b + cdot<i>(pxb, pyb, pzb);
    });
}

template <typename S>
__device__ __forceinline__ void cell_force_any(const StepArgs& a, uint32_t n, float& Fx, float& Fy,
                                               float& Fz) {
    Fx = a.fx; Fy = a.fy; Fz = a.fz;
    if (a.ffield != nullptr) {
        Fx = a.fx + a.ffield[n];
        Fy = a.fy + a.ffield[a.ffield_plane + n];
        Fz = a.fz + a.ffield[2u * a.ffield_plane + n];
    }
}

// The solid-fraction gradient is summed in FP64: a cell's per-step terms can
// be far larger than their sum over a long window (inside a fully solid body
// the adjoint is bounced without damping and grows with the window), and an
// FP32 running sum would lose the result's leading digits. Only cells with a
// solid fraction touch the array, so the FP64 adds cost nothing measurable.
__device__ __forceinline__ void add_grads(const AdjArgs& g, uint32_t n, float eps, float epsb,
                                          float Fbx, float Fby, float Fbz) {
    if (g.grad_eps != nullptr && eps != 0.0f) g.grad_eps[n] += double(epsb);
    if (g.grad_f != nullptr) {
        const uint32_t N = g.a.ffield_plane;
        g.grad_f[n] += Fbx;
        g.grad_f[N + n] += Fby;
        g.grad_f[2u * N + n] += Fbz;
    }
}

// One cell of the reverse even (in-cell) pass.
template <typename S, int GEO, bool LES>
__device__ __forceinline__ void adj_even_cell(const AdjArgs& g, int x, int y, int z) {
    const StepArgs& a = g.a;
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    float eps = 0.0f;
    if constexpr (GEO) {
        const uint8_t c = a.cell[n];
        if (c & CELL_TYPE_MASK) return;
        if (c & CELL_EPS_BIT) eps = a.eps[n];
    }
    const S* f = static_cast<const S*>(a.f);
    const uint64_t P = a.plane;
    float fh[19], ab[19];
    sfor<0, 19>([&](auto I) {
        fh[I] = load_ddf<S>(f + uint64_t(I) * P + n);
        ab[I] = g.lam[uint64_t(opp(I)) * P + n];
    });
    float Fx, Fy, Fz;
    cell_force_any<S>(a, n, Fx, Fy, Fz);
    float epsb, Fbx, Fby, Fbz;
    collide_adj<LES, GEO != 0>(fh, a, x, eps, Fx, Fy, Fz, ab, 0.f, 0.f, 0.f, g.force_terms != 0,
                               epsb, Fbx, Fby,
                Fbz);
    sfor<0, 19>([&](auto I) { g.lam[uint64_t(I) * P + n] = ab[I]; });
    add_grads(g, n, eps, epsb, Fbx, Fby, Fbz);
}

// One cell of the reverse odd (streaming) pass.
template <typename S, int GEO, bool LES>
__device__ __forceinline__ void adj_odd_cell(const AdjArgs& g, int x, int y, int z) {
    const StepArgs& a = g.a;
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    uint32_t geo = 0, lm = 0;
    float eps = 0.0f;
    if constexpr (GEO) {
        geo = a.geo[n];
        if (geo & GEO_NONFLUID) return;
        if (geo & GEO_EPS) eps = a.eps[n];
        if (geo & GEO_MOVING) lm = a.lmask[n];
    }
    const uint32_t wb = geo & GEO_WALL_BITS;
    const NbrOffsets nb(x, y, z, a.nx, a.ny, a.nz);
    const S* f = static_cast<const S*>(a.f);
    const uint64_t P = a.plane;
    const WallVel wv(a);
    // forward gather (Kernels.metal:272-314)
    float fh[19];
    uint32_t outflow_src = 0;  // loads negated by the dormant anti-bounce-back
    fh[0] = load_ddf<S>(f + n);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        const uint32_t src = uint32_t(int(n) + nb.template off<-dcx(i), -dcy(i), -dcz(i)>());
        const bool bb = (wb >> (o - 1)) & 1u;
        fh[i] = load_ddf<S>(f + (bb ? (uint64_t(i) * P + n) : (uint64_t(o) * P + src)));
        if (bb && ((lm >> (o - 1)) & 1u)) {
            const int sy = (y - dcy(i) + a.ny) % a.ny;
            const uint32_t s = (uint32_t((z - dcz(i) + a.nz) % a.nz) * uint32_t(a.ny) + uint32_t(sy)) *
                                   uint32_t(a.nx) +
                               uint32_t((x - dcx(i) + a.nx) % a.nx);
            const uint8_t wf = a.cell[s] & CELL_TYPE_MASK;
            if (wf == CELL_OUTFLOW) {
                fh[i] = -fh[i];
                outflow_src |= 1u << i;
            } else {
                float uwx, uwy, uwz;
                wall_velocity(wf, sy, a, wv, uwx, uwy, uwz);
                fh[i] += 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
            }
        }
    });
    float Fx, Fy, Fz;
    cell_force_any<S>(a, n, Fx, Fy, Fz);
    const bool obj = g.obj_w != 0.0f && (wb != 0u || eps > 0.0f) && x >= g.box[0] &&
                     x <= g.box[1] && y >= g.box[2] && y <= g.box[3];
    const float sx = obj ? g.obj_w * g.dir[0] : 0.f, sy_ = obj ? g.obj_w * g.dir[1] : 0.f,
                sz = obj ? g.obj_w * g.dir[2] : 0.f;
    // adjoints of the written values (Kernels.metal:317-350)
    float ab[19];
    ab[0] = g.lam[n];
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        const bool bb = (wb >> (i - 1)) & 1u;
        if (!bb) {
            const uint32_t dst = uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>());
            ab[i] = g.lam[uint64_t(i) * P + dst];
        } else {
            float sign = 1.0f;
            if ((lm >> (i - 1)) & 1u) {
                const uint32_t d = (uint32_t((z + dcz(i) + a.nz) % a.nz) * uint32_t(a.ny) +
                                    uint32_t((y + dcy(i) + a.ny) % a.ny)) *
                                       uint32_t(a.nx) +
                                   uint32_t((x + dcx(i) + a.nx) % a.nx);
                if ((a.cell[d] & CELL_TYPE_MASK) == CELL_OUTFLOW) sign = -1.0f;
            }
            // written value sign * fh'_i - corr; store-side force c_i (sign fh'_i + 2 w_i)
            ab[i] = sign * (g.lam[uint64_t(o) * P + n] + cdot<i>(sx, sy_, sz));
        }
    });
    float epsb, Fbx, Fby, Fbz;
    collide_adj<LES, GEO != 0>(fh, a, x, eps, Fx, Fy, Fz, ab, sx, sy_, sz, g.force_terms != 0,
                               epsb, Fbx, Fby,
                Fbz);
    // back to the slots that were read; load-side force -c_i * (raw load)
    g.lam[n] = ab[0];
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        const bool bb = (wb >> (o - 1)) & 1u;
        if (bb) {
            float v = ((outflow_src >> i) & 1u) ? -ab[i] : ab[i];
            v -= cdot<i>(sx, sy_, sz);
            g.lam[uint64_t(i) * P + n] = v;
        } else {
            const uint32_t src = uint32_t(int(n) + nb.template off<-dcx(i), -dcy(i), -dcz(i)>());
            g.lam[uint64_t(o) * P + src] = ab[i];
        }
    });
    add_grads(g, n, eps, epsb, Fbx, Fby, Fbz);
}

// Block of a block list: block i of the grid processes lattice block list[i]
// (linear index bx + gx * (by + gy * bz)) of the (blockDim.x, blockDim.y) grid.
__device__ __forceinline__ void adj_list_block(const uint32_t* list, uint32_t gx, uint32_t gy,
                                               int& x, int& y, int& z) {
    const uint32_t blk = list[blockIdx.x];
    const uint32_t t = blk / gx;
    x = int((blk - t * gx) * blockDim.x + threadIdx.x);
    y = int((t % gy) * blockDim.y + threadIdx.y);
    z = int(t / gy);
}

template <typename S, int GEO, bool LES>
__global__ void __launch_bounds__(128) k_adj_even(const AdjArgs g) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= g.a.nx || y >= g.a.ny) return;
    adj_even_cell<S, GEO, LES>(g, x, y, blockIdx.z);
}

// At least four resident blocks: left to itself the compiler gives the odd
// adjoint 184 registers (two blocks of 128 threads per SM, 12% of the warp
// slots, IPC 1.0); capped at 128 (a few spilled words) the reverse step of
// the cylinder runs in 1.78x a forward step instead of 2.20x. Without walls
// and LES the reverse step fits 96 registers (five blocks per SM; FP16 storage
// spills a few words).
template <int GEO, bool LES>
constexpr int adj_odd_min_blocks() {
    return (GEO == 0 && !LES) ? 5 : 4;
}

template <typename S, int GEO, bool LES>
__global__ void __launch_bounds__(128, adj_odd_min_blocks<GEO, LES>()) k_adj_odd(const AdjArgs g) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= g.a.nx || y >= g.a.ny) return;
    adj_odd_cell<S, GEO, LES>(g, x, y, blockIdx.z);
}

// Block-list forms for the bulk / boundary split of a walled lattice: the
// bulk blocks (no wall, no wall neighbour, no solid fraction) take the
// wall-free reverse step, the boundary blocks the wall-aware one, as in the
// forward split. The per-cell values are the same as the grid forms'.
template <typename S, int GEO, bool LES>
__global__ void __launch_bounds__(128) k_adj_list_even(const AdjArgs g, const uint32_t* list,
                                                       uint32_t gx, uint32_t gy) {
    int x, y, z;
    adj_list_block(list, gx, gy, x, y, z);
    if (x >= g.a.nx || y >= g.a.ny || z >= g.a.nz) return;
    adj_even_cell<S, GEO, LES>(g, x, y, z);
}

template <typename S, int GEO, bool LES>
__global__ void __launch_bounds__(128, adj_odd_min_blocks<GEO, LES>()) k_adj_list_odd(const AdjArgs g, const uint32_t* list,
                                                         uint32_t gx, uint32_t gy) {
    int x, y, z;
    adj_list_block(list, gx, gy, x, y, z);
    if (x >= g.a.nx || y >= g.a.ny || z >= g.a.nz) return;
    adj_odd_cell<S, GEO, LES>(g, x, y, z);
}

template <typename S, int GEO, bool LES>
void launch_adj_list_les(const AdjArgs& g, int parity, const uint32_t* list, uint32_t count,
                         dim3 block, cudaStream_t st) {
    const uint32_t gx = (uint32_t(g.a.nx) + block.x - 1) / block.x;
    const uint32_t gy = (uint32_t(g.a.ny) + block.y - 1) / block.y;
    if (parity == 0) k_adj_list_even<S, GEO, LES><<<count, block, 0, st>>>(g, list, gx, gy);
    else k_adj_list_odd<S, GEO, LES><<<count, block, 0, st>>>(g, list, gx, gy);
}

template <typename S, int GEO>
void launch_adj_list(const AdjArgs& g, int parity, const uint32_t* list, uint32_t count,
                     dim3 block, cudaStream_t st) {
    if (count == 0) return;
    if (g.a.c_smago > 0.0f) launch_adj_list_les<S, GEO, true>(g, parity, list, count, block, st);
    else launch_adj_list_les<S, GEO, false>(g, parity, list, count, block, st);
}

// Gradient of the dissipation objective at one sampled state. Per fluid cell,
// with u = (p + F/2) / rho, Pi the non-equilibrium second moment and
// s = 1.5 omega / rho, the cell's term 2 nu s^2 Pi:Pi has
//   d/df_j = 4 nu s^2 [ (c_j - u).Pi.(c_j - u) - tr(Pi) / 3 - Pi:Pi / rho ],
//   d/dF   = -4 nu s^2 Pi u,
// because Pi_ab = sum_i c_ia c_ib f_i - (rho - 1) / 3 delta_ab - rho u_a u_b
// (the D3Q19 equilibrium's second moment), so dPi_ab/df_j = (c_ja - u_a)
// (c_jb - u_b) - delta_ab / 3, and s^2 falls with rho as -2 s^2 / rho. Pi
// itself is summed direction by direction as the observable does.
template <typename S>
__global__ void __launch_bounds__(128) k_adj_dissipation(const AdjArgs g, float nu, float w) {
    const StepArgs& a = g.a;
    const uint64_t N = uint64_t(a.nx) * uint64_t(a.ny) * uint64_t(a.nz);
    const S* __restrict__ f = static_cast<const S*>(a.f);
    const uint64_t P = a.plane;
    for (uint64_t n = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; n < N;
         n += uint64_t(gridDim.x) * blockDim.x) {
        if (a.cell != nullptr && (a.cell[n] & CELL_TYPE_MASK) != CELL_FLUID) continue;
        float fh[19];
        sfor<0, 19>([&](auto I) { fh[I] = load_ddf<S>(f + uint64_t(I) * P + n); });
        float rhom1 = fh[0];
        sfor<1, 19>([&](auto I) { rhom1 += fh[I]; });
        float px = 0.f, py = 0.f, pz = 0.f;
        sfor<1, 19>([&](auto I) { add_c<I>(px, py, pz, fh[I]); });
        float Fx, Fy, Fz;
        cell_force_any<S>(a, uint32_t(n), Fx, Fy, Fz);
        const float rho = 1.0f + rhom1;
        const float ux = (px + 0.5f * Fx) / rho, uy = (py + 0.5f * Fy) / rho,
                    uz = (pz + 0.5f * Fz) / rho;
        const float u2 = ux * ux + uy * uy + uz * uz;
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
        const float sc = 1.5f * a.omega / rho;
        const float k4 = w * 4.0f * nu * sc * sc;
        const float base = -(pxx + pyy + pzz) * (1.0f / 3.0f) - pipi / rho;
        sfor<0, 19>([&](auto I) {
            constexpr int i = I;
            const float ex = float(dcx(i)) - ux, ey = float(dcy(i)) - uy, ez = float(dcz(i)) - uz;
            const float q = ex * ex * pxx + ey * ey * pyy + ez * ez * pzz +
                            2.0f * (ex * ey * pxy + ex * ez * pxz + ey * ez * pyz);
            g.lam[uint64_t(i) * P + n] += k4 * (q + base);
        });
        if (g.grad_f != nullptr) {
            const uint64_t FP = g.a.ffield_plane;
            g.grad_f[n] -= k4 * (pxx * ux + pxy * uy + pxz * uz);
            g.grad_f[FP + n] -= k4 * (pxy * ux + pyy * uy + pyz * uz);
            g.grad_f[2 * FP + n] -= k4 * (pxz * ux + pyz * uy + pzz * uz);
        }
    }
}

}  // namespace

cudaError_t launch_adjoint_dissipation(const AdjArgs& g, int half_storage, float nu, float w,
                                       cudaStream_t st) {
    const uint64_t N = uint64_t(g.a.nx) * uint64_t(g.a.ny) * uint64_t(g.a.nz);
    const uint64_t want = (N + 127) / 128;
    const unsigned blocks = unsigned(want < 152u * 64u ? want : 152u * 64u);
    if (half_storage) k_adj_dissipation<__half><<<blocks, 128, 0, st>>>(g, nu, w);
    else k_adj_dissipation<float><<<blocks, 128, 0, st>>>(g, nu, w);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_split(const AdjArgs& g, int half_storage, int parity, dim3 block,
                                 const uint32_t* bulk, uint32_t nbulk, const uint32_t* edge,
                                 uint32_t nedge, cudaStream_t st) {
    if (block.x * block.y > 128) return cudaErrorInvalidValue;
    if (half_storage) {
        launch_adj_list<__half, 0>(g, parity, bulk, nbulk, block, st);
        launch_adj_list<__half, 1>(g, parity, edge, nedge, block, st);
    } else {
        launch_adj_list<float, 0>(g, parity, bulk, nbulk, block, st);
        launch_adj_list<float, 1>(g, parity, edge, nedge, block, st);
    }
    return cudaGetLastError();
}

template <typename S, bool LES>
static void launch_adj_grid(const AdjArgs& g, int parity, int geo, dim3 grid, dim3 block,
                            cudaStream_t st) {
    if (parity == 0) {
        if (geo) k_adj_even<S, 1, LES><<<grid, block, 0, st>>>(g);
        else k_adj_even<S, 0, LES><<<grid, block, 0, st>>>(g);
    } else {
        if (geo) k_adj_odd<S, 1, LES><<<grid, block, 0, st>>>(g);
        else k_adj_odd<S, 0, LES><<<grid, block, 0, st>>>(g);
    }
}

cudaError_t launch_adjoint_step(const AdjArgs& g, int half_storage, int parity, int geo, dim3 block,
                                cudaStream_t st) {
    const dim3 grid((g.a.nx + block.x - 1) / block.x, (g.a.ny + block.y - 1) / block.y, g.a.nz);
    const bool les = g.a.c_smago > 0.0f;
    if (half_storage) {
        if (les) launch_adj_grid<__half, true>(g, parity, geo, grid, block, st);
        else launch_adj_grid<__half, false>(g, parity, geo, grid, block, st);
    } else {
        if (les) launch_adj_grid<float, true>(g, parity, geo, grid, block, st);
        else launch_adj_grid<float, false>(g, parity, geo, grid, block, st);
    }
    return cudaGetLastError();
}

}  // namespace stro
