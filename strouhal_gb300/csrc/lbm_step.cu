// The D3Q19 AA-pattern fused stream-collide step for sm_103a.
//
// Restates the reference's `step` kernel (Kernels.metal:230-355) and its
// `collide` (Kernels.metal:105-228) as two kernels, one per AA parity:
//   even: read slot i of cell n, collide, write slot opp(i) of cell n;
//   odd : read slot opp(i) of n - c_i (or slot i of n behind a wall), collide,
//         write slot i of n + c_i (or slot opp(i) of n toward a wall).
// Each slot has one reader and one writer per pass and they are the same
// thread, so the update is in place and race-free with no atomics.
//
// Arithmetic contract: this file is compiled with -fmad=false and the only
// fused multiply-add is the explicit one of the reference (Kernels.metal:181),
// divisions and square roots are IEEE-rounded, and every expression keeps the
// reference's operation order. The results are therefore equal in value to
// the reference arithmetic evaluated in FP32 (only zero terms are skipped).
//
// Specialisations (all value-preserving):
//   GEO  = 0 periodic all-fluid box: no cell bytes, masks or wall logic;
//          1 walls and/or partially saturated cells.
//   FEAT = 0 lean collide: no sponge, LES, body force or NT cells;
//          1 all features, each behind a uniform or per-cell branch.
//   PROBE  odd pass with momentum-exchange force accumulation, reduced per
//          block in FP64 in a fixed order (no per-cell force buffer).
#include "lbm_device.cuh"
#include "lbm_launch.h"

namespace stro {

__device__ __forceinline__ int wrapi(int v, int n) {  // Kernels.metal:73-77
    v += (v < 0) ? n : 0;
    v -= (v >= n) ? n : 0;
    return v;
}

// Wall velocity of a moving-wall cell at row wy, Kernels.metal:79-87.
__device__ __forceinline__ void wall_velocity(uint8_t wf, int wy, const StepArgs& a, float& ux,
                                              float& uy, float& uz) {
    if (wf == CELL_LID) {
        ux = a.ulid_x; uy = a.ulid_y; uz = a.ulid_z;
        return;
    }
    uy = 0.0f; uz = 0.0f;
    if (a.inflow_uniform != 0) { ux = a.uin; return; }
    const float H = (float)a.ny - 2.0f;
    const float yd = (float)wy - 0.5f;
    ux = fmaxf(4.0f * a.uin * yd * (H - yd) / (H * H), 0.0f);
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

// Collision, Kernels.metal:105-228.
template <bool FEAT>
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
    float ux, uy, uz;
    if constexpr (FEAT) {
        ux = (px + 0.5f * Fx) * inv;
        uy = (py + 0.5f * Fy) * inv;
        uz = (pz + 0.5f * Fz) * inv;
    } else {
        ux = px * inv;
        uy = py * inv;
        uz = pz * inv;
    }
    const float u2 = ux * ux + uy * uy + uz * uz;

    if constexpr (FEAT) {
        if (a.c_smago > 0.0f) {  // Smagorinsky LES, Kernels.metal:140-167
            float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
            sfor<1, 19>([&](auto I) {
                constexpr int i = I;
                constexpr float w = wgt(i);
                const float cu = 3.0f * cdot<i>(ux, uy, uz);
                const float feq = w * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
                const float d = fh[i] - feq;
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
            const float Q = sqrtf(pxx * pxx + pyy * pyy + pzz * pzz +
                                  2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
            const float tau0 = 1.0f / wp;
            const float tauEff =
                0.5f * (tau0 + sqrtf(tau0 * tau0 + 25.455844f * a.c_smago * Q * inv));
            if (a.omega_minus == a.omega) {
                wp = 1.0f / tauEff;
                wm = wp;
            } else {
                const float lambda = (1.0f / wp - 0.5f) * (1.0f / wm - 0.5f);
                wp = 1.0f / tauEff;
                wm = 1.0f / (0.5f + lambda / (tauEff - 0.5f));
            }
        }
        if (eps == 0.0f) {
            if (a.force_on) relax<true, false>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty, ntz);
            else relax<false, false>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty, ntz);
        } else {
            if (a.force_on) relax<true, true>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty, ntz);
            else relax<false, true>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, Fx, Fy, Fz, eps, ntx, nty, ntz);
        }
    } else {
        relax<false, false>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, 0.f, 0.f, 0.f, 0.f, ntx, nty, ntz);
    }
}

template <bool FEAT>
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

// ---------------------------------------------------------------- even pass
template <typename S, int GEO, bool FEAT>
__global__ void __launch_bounds__(256) k_step_even(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= a.nx || y >= a.ny) return;
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    float eps = 0.0f;
    if constexpr (GEO) {
        const uint8_t c = a.cell[n];
        if (c & CELL_TYPE_MASK) return;
        if constexpr (FEAT) {
            if (c & CELL_EPS_BIT) eps = a.eps[n];
        }
    }
    S* __restrict__ f = static_cast<S*>(a.f);
    const uint64_t P = a.plane;
    float fh[19];
    sfor<0, 19>([&](auto I) { fh[I] = load_ddf<S>(f + uint64_t(I) * P + n); });
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT>(fh, a, x, eps, Fx, Fy, Fz, ntx, nty, ntz);
    store_ddf<S>(f + n, fh[0]);
    sfor<1, 19>([&](auto I) { store_ddf<S>(f + uint64_t(opp(I)) * P + n, fh[I]); });
}

// Deferred moving-wall corrections of the gathered DDFs, Kernels.metal:292-314.
template <bool PROBE>
__device__ __forceinline__ void moving_wall_loads(float (&fh)[19], const StepArgs& a, uint32_t wb,
                                               uint32_t lm, int x, int y, int z, float& ax,
                                               float& ay, float& az) {
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
            } else {
                float uwx, uwy, uwz;
                wall_velocity(wf, sy, a, uwx, uwy, uwz);
                const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                fh[i] += corr;
                if constexpr (PROBE) acc_sub<i>(ax, ay, az, corr);
            }
        }
    });
}

// Scatter with moving-wall corrections, Kernels.metal:317-350.
template <typename S, bool PROBE>
__device__ __forceinline__ void moving_wall_stores(const float (&fh)[19], const StepArgs& a,
                                                uint32_t n, uint32_t wb, uint32_t lm, int x, int y,
                                                int z, const NbrOffsets& nb, float& ax, float& ay,
                                                float& az) {
    S* __restrict__ f = static_cast<S*>(a.f);
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
                    out = sv;
                } else {
                    float uwx, uwy, uwz;
                    wall_velocity(wf, dy, a, uwx, uwy, uwz);
                    const float corr = 6.0f * wgt(i) * cdot<i>(uwx, uwy, uwz);
                    out = sv - corr;
                }
            }
            store_ddf<S>(f + uint64_t(opp(i)) * P + n, out);
            if constexpr (PROBE) acc_add<i>(ax, ay, az, sv + 2.0f * wgt(i));
        }
    });
}

// ----------------------------------------------------------------- odd pass
template <typename S, int GEO, bool FEAT, bool PROBE>
__global__ void __launch_bounds__(256) k_step_odd(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    double contrib[3] = {0.0, 0.0, 0.0};
    bool active = (x < a.nx && y < a.ny);
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    uint32_t g = 0;
    if constexpr (GEO) {
        if (active) {
            g = a.geo[n];
            if (g & GEO_NONFLUID) active = false;
        }
    }
    if constexpr (!PROBE) {
        if (!active) return;
    }
    if (active) {
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
        fh[0] = load_ddf<S>(f + n);
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            constexpr int o = opp(i);
            const uint32_t src = uint32_t(int(n) + nb.template off<-dcx(i), -dcy(i), -dcz(i)>());
            if constexpr (GEO) {
                const bool bb = (wb >> (o - 1)) & 1u;
                const uint64_t idx = bb ? (uint64_t(i) * P + n) : (uint64_t(o) * P + src);
                fh[i] = load_ddf<S>(f + idx);
                if constexpr (PROBE) {
                    if (bb) acc_sub<i>(ax, ay, az, fh[i]);
                }
            } else {
                fh[i] = load_ddf<S>(f + uint64_t(o) * P + src);
            }
        });
        uint32_t lm = 0;
        if constexpr (GEO) {
            if (g & GEO_MOVING) {
                lm = a.lmask[n];
                moving_wall_loads<PROBE>(fh, a, wb, lm, x, y, z, ax, ay, az);
            }
        }
        float Fx = 0.f, Fy = 0.f, Fz = 0.f;
        cell_force<FEAT>(a, n, Fx, Fy, Fz);
        float ntx = 0.f, nty = 0.f, ntz = 0.f;
        collide<FEAT>(fh, a, x, eps, Fx, Fy, Fz, ntx, nty, ntz);
        if constexpr (PROBE) {
            ax += ntx;
            ay += nty;
            az += ntz;
        }
        store_ddf<S>(f + n, fh[0]);
        if constexpr (GEO) {
            if (!(g & GEO_MOVING)) {
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
                moving_wall_stores<S, PROBE>(fh, a, n, wb, lm, x, y, z, nb, ax, ay, az);
            }
        } else {
            sfor<1, 19>([&](auto I) {
                constexpr int i = I;
                const uint32_t dst = uint32_t(int(n) + nb.template off<dcx(i), dcy(i), dcz(i)>());
                store_ddf<S>(f + uint64_t(i) * P + dst, fh[i]);
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
    if constexpr (PROBE) {
        const uint32_t blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        block_reduce_store<3>(contrib, a.partials + 3u * blk);
    }
}

// ----------------------------------------------------------------- launcher
template <typename S>
static cudaError_t launch_typed(const StepArgs& a, int parity, int geo, bool feat, bool probe,
                                dim3 grid, dim3 block, cudaStream_t st) {
    if (parity == 0) {
        if (geo) {
            if (feat) k_step_even<S, 1, true><<<grid, block, 0, st>>>(a);
            else k_step_even<S, 1, false><<<grid, block, 0, st>>>(a);
        } else {
            if (feat) k_step_even<S, 0, true><<<grid, block, 0, st>>>(a);
            else k_step_even<S, 0, false><<<grid, block, 0, st>>>(a);
        }
    } else {
        if (probe) {
            if (!geo) return cudaErrorInvalidValue;
            if (feat) k_step_odd<S, 1, true, true><<<grid, block, 0, st>>>(a);
            else k_step_odd<S, 1, false, true><<<grid, block, 0, st>>>(a);
        } else if (geo) {
            if (feat) k_step_odd<S, 1, true, false><<<grid, block, 0, st>>>(a);
            else k_step_odd<S, 1, false, false><<<grid, block, 0, st>>>(a);
        } else {
            if (feat) k_step_odd<S, 0, true, false><<<grid, block, 0, st>>>(a);
            else k_step_odd<S, 0, false, false><<<grid, block, 0, st>>>(a);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_step(const StepArgs& a, int half_storage, int parity, int geo, bool feat,
                        bool probe, dim3 block, cudaStream_t st) {
    const dim3 grid((a.nx + block.x - 1) / block.x, (a.ny + block.y - 1) / block.y, a.nz);
    if (half_storage) return launch_typed<__half>(a, parity, geo, feat, probe, grid, block, st);
    return launch_typed<float>(a, parity, geo, feat, probe, grid, block, st);
}

dim3 step_grid(const StepArgs& a, dim3 block) {
    return dim3((a.nx + block.x - 1) / block.x, (a.ny + block.y - 1) / block.y, a.nz);
}

}  // namespace stro
