// CPU oracle for the D3Q19 AA stream-collide step — TEST INFRASTRUCTURE ONLY.
//
// A scalar restatement of the reference's Metal kernel arithmetic
// (Sources/StrouhalCore/Kernels.metal) and of the host-side set-up in
// Sources/StrouhalCore/Sim.swift, templated on the arithmetic type Real and the
// DDF storage type Store:
//   <float, float>     value-identical to the reference kernel at FPXX=float
//   <float, _Float16>  value-identical to the reference kernel at FPXX=half
//   <double, double>   the FP64 oracle (same algorithm, double throughout)
// and, with FUSED, the library's fused-multiply-add arithmetic (an
// algebraically equal form of the same collision that the reference does not
// have): kinds 3 and 4 below, FP32 arithmetic over FP32 and FP16 storage.
// "Value-identical" means equal as IEEE numbers (+0 == -0): terms whose lattice
// coefficient is 0 are skipped, which can only change the sign of a zero.
// The <float,*> instances are pinned against the reference's own kernel source
// compiled as C++ (oracle/ref_metal_driver.cpp) by tests/test_oracle_pin.py.
//
// Only tests/, the smoke check and bench.py's CPU-baseline leg load this
// library. Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp (oracle/build_oracle.py).
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// D3Q19 velocity set and pairing, Kernels.metal:38-47 (order is load-bearing:
// opp(i) = i odd ? i+1 : i-1).
const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

enum : uint8_t { FLUID = 0, SOLID = 1, LID = 2, INFLOW = 3, OUTFLOW = 4 };

// Per-step uniforms, byte layout of Kernels.metal:49-63 / Sim.swift:10-24.
struct Params {
    uint32_t nx, ny, nz, parity;
    float omega, omegaMinus, uin, cSmago;
    float fx, fy, fz;
    uint32_t writeForce;
    float ulidX, ulidY, ulidZ;
    uint32_t inflowUniform;
    float spongeX0, spongeInvW, spongeTau;
    uint32_t useEps;
};
static_assert(sizeof(Params) == 80, "Params layout");

// Options of the library's extensions, outside the reference's Params.
constexpr int OPT_PRESSURE_OUTFLOW = 1;
constexpr int OPT_KBC = 2;

// Math through unqualified calls, so a dual-number type can supply its own.
using std::fma;
using std::fmax;
using std::fmin;
using std::sqrt;
template <class R> inline R Sqrt(R a) { return sqrt(a); }
template <class R> inline R Fma(R a, R b, R c) { return fma(a, b, c); }
template <class R> inline R Fmin(R a, R b) { return fmin(a, b); }
template <class R> inline R Fmax(R a, R b) { return fmax(a, b); }

// Forward-mode dual number with K derivative lanes, in double. Instantiating
// the restated kernel arithmetic on it gives the exact local Jacobian of a
// cell update (used by the FP64 adjoint below).
template <int K> struct Dual {
    double v;
    double d[K];
    Dual() : v(0.0) { for (int k = 0; k < K; ++k) d[k] = 0.0; }
    Dual(double x) : v(x) { for (int k = 0; k < K; ++k) d[k] = 0.0; }  // NOLINT: implicit
    static Dual var(double x, int lane) {
        Dual r(x);
        r.d[lane] = 1.0;
        return r;
    }
};
template <int K> inline Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v + b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K> inline Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v - b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K> inline Dual<K> operator-(const Dual<K>& a) {
    Dual<K> r(-a.v);
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int K> inline Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v * b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K> inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v / b.v);
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
template <int K> inline Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b) { return a = a + b; }
template <int K> inline Dual<K>& operator-=(Dual<K>& a, const Dual<K>& b) { return a = a - b; }
template <int K> inline bool operator==(const Dual<K>& a, const Dual<K>& b) { return a.v == b.v; }
template <int K> inline bool operator>(const Dual<K>& a, const Dual<K>& b) { return a.v > b.v; }
template <int K> inline bool operator<(const Dual<K>& a, const Dual<K>& b) { return a.v < b.v; }
template <int K> inline Dual<K> sqrt(const Dual<K>& a) {
    Dual<K> r(std::sqrt(a.v));
    const double g = r.v > 0.0 ? 0.5 / r.v : 0.0;  // subgradient 0 at the kink
    for (int k = 0; k < K; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int K> inline Dual<K> fma(const Dual<K>& a, const Dual<K>& b, const Dual<K>& c) {
    return a * b + c;
}
template <int K> inline Dual<K> fmin(const Dual<K>& a, const Dual<K>& b) { return b.v < a.v ? b : a; }
template <int K> inline Dual<K> fmax(const Dual<K>& a, const Dual<K>& b) { return b.v > a.v ? b : a; }

template <class R> inline R weight(int i) {
    return i == 0 ? R(1) / R(3) : (i < 7 ? R(1) / R(18) : R(1) / R(36));
}
template <class R> inline R smagConst() { return R(18.0 * std::sqrt(2.0)); }  // Kernels.metal:156-157
template <> inline float smagConst<float>() { return 25.455844f; }

// sum_k c_k * v_k over the three components, in x,y,z order, skipping zero
// coefficients (value-identical to the reference's (float)Cx*vx + ... form).
template <class R> inline R cdot(int i, R vx, R vy, R vz) {
    R s = R(0);
    bool any = false;
    const int c[3] = {CX[i], CY[i], CZ[i]};
    const R v[3] = {vx, vy, vz};
    for (int k = 0; k < 3; ++k) {
        if (c[k] == 0) continue;
        const R t = c[k] > 0 ? v[k] : -v[k];
        s = any ? s + t : t;
        any = true;
    }
    return s;
}

inline int wrap(int v, int n) {  // Kernels.metal:73-77
    v += (v < 0) ? n : 0;
    v -= (v >= n) ? n : 0;
    return v;
}

template <class R> struct V3 { R x, y, z; };

// Wall velocity of a moving-wall cell, Kernels.metal:79-87.
template <class R> inline V3<R> wall_velocity(uint8_t wf, int wy, const Params& p) {
    if (wf == LID) return {R(p.ulidX), R(p.ulidY), R(p.ulidZ)};
    if (p.inflowUniform != 0u) return {R(p.uin), R(0), R(0)};
    const R H = R(p.ny) - R(2);
    const R yd = R(wy) - R(0.5);
    const R prof = R(4) * R(p.uin) * yd * (H - yd) / (H * H);
    return {Fmax(prof, R(0)), R(0), R(0)};
}

// TRT + Guo + sponge + Smagorinsky + Noble-Torczynski collision on shifted
// DDFs, Kernels.metal:105-228. F is the cell's body force (the reference's
// uniform force plus the optional per-cell field extension).
template <class R>
void relax_fused(R* fh, R wp, R wm, R rho, R rhom1, R ux, R uy, R uz, R u2, const R F[3], R eps,
                 R nt[3]);

template <class R>
void relax_kbc(R* fh, R w, R rho, R rhom1, R ux, R uy, R uz, R u2, const R F[3], bool force);

template <class R, bool FUSED = false>
void collide(R* fh, const Params& p, int x, R eps, const R F[3], R& rhoOut, R nt[3],
             bool kbc = false) {
    R wp = R(p.omega), wm = R(p.omegaMinus);
    if (R(x) > R(p.spongeX0)) {  // sponge, Kernels.metal:112-123
        const R frac = Fmin((R(x) - R(p.spongeX0)) * R(p.spongeInvW), R(1));
        const R tau0 = R(1) / wp;
        const R tauS = tau0 + frac * (R(p.spongeTau) - tau0);
        if (p.omegaMinus == p.omega) {
            wp = R(1) / tauS;
            wm = wp;
        } else {
            const R lambda = (R(1) / wp - R(0.5)) * (R(1) / wm - R(0.5));
            wp = R(1) / tauS;
            wm = R(1) / (R(0.5) + lambda / (tauS - R(0.5)));
        }
    }
    // moments, Kernels.metal:124-138
    R rhom1 = fh[0];
    for (int i = 1; i < 19; ++i) rhom1 += fh[i];
    const R rho = R(1) + rhom1;
    rhoOut = rho;
    const R inv = R(1) / rho;
    R pc[3] = {R(0), R(0), R(0)};
    bool started[3] = {false, false, false};
    for (int i = 1; i < 19; ++i) {
        const int c[3] = {CX[i], CY[i], CZ[i]};
        for (int k = 0; k < 3; ++k) {
            if (c[k] == 0) continue;
            const R t = c[k] > 0 ? fh[i] : -fh[i];
            pc[k] = started[k] ? pc[k] + t : t;
            started[k] = true;
        }
    }
    R ux, uy, uz, u2;
    if (!FUSED) {
        ux = (pc[0] + R(0.5) * F[0]) * inv;
        uy = (pc[1] + R(0.5) * F[1]) * inv;
        uz = (pc[2] + R(0.5) * F[2]) * inv;
        u2 = ux * ux + uy * uy + uz * uz;
    } else {
        ux = Fma(R(0.5), F[0], pc[0]) * inv;
        uy = Fma(R(0.5), F[1], pc[1]) * inv;
        uz = Fma(R(0.5), F[2], pc[2]) * inv;
        u2 = Fma(uz, uz, Fma(uy, uy, ux * ux));
    }
    if (kbc) {  // the KBC collision: sponge and force only (the library refuses LES and NT)
        const R u2k = ux * ux + uy * uy + uz * uz;
        const bool force = !(F[0] == R(0)) || !(F[1] == R(0)) || !(F[2] == R(0));
        relax_kbc<R>(fh, wp, rho, rhom1, ux, uy, uz, u2k, F, force);
        return;
    }

    if (R(p.cSmago) > R(0)) {  // Smagorinsky, Kernels.metal:140-167
        R pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
        bool sxx = false, syy = false, szz = false, sxy = false, sxz = false, syz = false;
        auto acc = [](R& a, bool& s, int coef, R d) {
            if (coef == 0) return;
            const R t = coef > 0 ? d : -d;
            a = s ? a + t : t;
            s = true;
        };
        for (int i = 1; i < 19; ++i) {
            R d = fh[i];  // fused: raw second moments, the equilibrium's are subtracted below
            if (!FUSED) {
                const R cu = R(3) * cdot<R>(i, ux, uy, uz);
                const R feq =
                    weight<R>(i) * (rhom1 + rho * (cu + R(0.5) * cu * cu - R(1.5) * u2));
                d = fh[i] - feq;
            }
            acc(pxx, sxx, CX[i] * CX[i], d);
            acc(pyy, syy, CY[i] * CY[i], d);
            acc(pzz, szz, CZ[i] * CZ[i], d);
            acc(pxy, sxy, CX[i] * CY[i], d);
            acc(pxz, sxz, CX[i] * CZ[i], d);
            acc(pyz, syz, CY[i] * CZ[i], d);
        }
        R Q, tauEff;
        const R tau0 = R(1) / wp;
        if (!FUSED) {
            Q = Sqrt(pxx * pxx + pyy * pyy + pzz * pzz + R(2) * (pxy * pxy + pxz * pxz + pyz * pyz));
            tauEff = R(0.5) * (tau0 + Sqrt(tau0 * tau0 + smagConst<R>() * R(p.cSmago) * Q * inv));
        } else {
            // sum_i c_ia c_ib feq_i = rhom1/3 delta_ab + rho u_a u_b for shifted DDFs
            const R r3 = rhom1 * (R(1) / R(3));
            const R rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
            pxx = Fma(-rux, ux, pxx - r3);
            pyy = Fma(-ruy, uy, pyy - r3);
            pzz = Fma(-ruz, uz, pzz - r3);
            pxy = Fma(-rux, uy, pxy);
            pxz = Fma(-rux, uz, pxz);
            pyz = Fma(-ruy, uz, pyz);
            Q = Sqrt(Fma(pzz, pzz, Fma(pyy, pyy, pxx * pxx)) +
                     R(2) * Fma(pyz, pyz, Fma(pxz, pxz, pxy * pxy)));
            tauEff = R(0.5) *
                     (tau0 + Sqrt(Fma(tau0, tau0, smagConst<R>() * R(p.cSmago) * Q * inv)));
        }
        if (p.omegaMinus == p.omega) {
            wp = R(1) / tauEff;
            wm = wp;
        } else {
            const R lambda = (R(1) / wp - R(0.5)) * (R(1) / wm - R(0.5));
            wp = R(1) / tauEff;
            wm = R(1) / (R(0.5) + lambda / (tauEff - R(0.5)));
        }
    }

    if (FUSED) {
        relax_fused<R>(fh, wp, wm, rho, rhom1, ux, uy, uz, u2, F, eps, nt);
        return;
    }
    const R uF = ux * F[0] + uy * F[1] + uz * F[2];
    const R ap = R(1) - R(0.5) * wp;
    const R am = R(1) - R(0.5) * wm;
    const R w0 = weight<R>(0);
    const R feq0 = w0 * (rhom1 - R(1.5) * rho * u2);
    const R s0 = w0 * ap * (R(-3) * uF);

    if (eps == R(0)) {  // Kernels.metal:177-199 (bit-compatible golden path)
        fh[0] = Fma(wp, feq0 - fh[0], fh[0]) + s0;
        for (int i = 1; i < 19; i += 2) {
            const R w = weight<R>(i);
            const R cu = R(3) * cdot<R>(i, ux, uy, uz);
            const R cF = cdot<R>(i, F[0], F[1], F[2]);
            const R feqp = w * (rhom1 + rho * (R(0.5) * cu * cu - R(1.5) * u2));
            const R feqm = w * rho * cu;
            const R fp = R(0.5) * (fh[i] + fh[i + 1]);
            const R fm = R(0.5) * (fh[i] - fh[i + 1]);
            const R dp = wp * (feqp - fp);
            const R dm = wm * (feqm - fm);
            const R sm = w * am * (R(3) * cF);
            const R sp = w * ap * (R(3) * cu * cF - R(3) * uF);
            fh[i] += dp + dm + sp + sm;
            fh[i + 1] += dp - dm + sp - sm;
        }
        return;
    }
    // Noble-Torczynski partially saturated cell, Kernels.metal:201-227
    const R tw = R(1) / wp - R(0.5);
    const R B = eps * tw / ((R(1) - eps) + tw);
    const R oneMinusB = R(1) - B;
    fh[0] += oneMinusB * (wp * (feq0 - fh[0]) + s0);
    for (int i = 1; i < 19; i += 2) {
        const R w = weight<R>(i);
        const R cu = R(3) * cdot<R>(i, ux, uy, uz);
        const R cF = cdot<R>(i, F[0], F[1], F[2]);
        const R feqp = w * (rhom1 + rho * (R(0.5) * cu * cu - R(1.5) * u2));
        const R feqm = w * rho * cu;
        const R fp = R(0.5) * (fh[i] + fh[i + 1]);
        const R fm = R(0.5) * (fh[i] - fh[i + 1]);
        const R dp = wp * (feqp - fp);
        const R dm = wm * (feqm - fm);
        const R sm = w * am * (R(3) * cF);
        const R sp = w * ap * (R(3) * cu * cF - R(3) * uF);
        const R bounce = B * (fh[i + 1] - fh[i]);
        fh[i] += oneMinusB * (dp + dm + sp + sm) + bounce;
        fh[i + 1] += oneMinusB * (dp - dm + sp - sm) - bounce;
        const int c[3] = {CX[i], CY[i], CZ[i]};
        for (int k = 0; k < 3; ++k)
            if (c[k] != 0) nt[k] -= R(2 * c[k]) * bounce;
    }
}

// The fused relaxation, operation for operation as the GPU's fused mode:
//   feq+ = fma(w rho, fma(4.5 cd, cd, -1.5 u2), w (rho-1)),  feq- = (w rho)(3 cd)
//   A = fma(-1/2, f_i + f_j, feq+),  B = fma(-1/2, f_i - f_j, feq-)
//   f_i' = fma(w+, A, fma(w-, B, f_i + (s+ + s-))),
//   f_j' = fma(w+, A, fma(-w-, B, f_j + (s+ - s-)))
// with cd = c_i . u, j = opp(i), s+/s- the split Guo source terms; partially
// saturated cells blend with the Noble-Torczynski bounce operator as in
// Kernels.metal:201-227. Same steps as relax_fused in lbm_cell.cuh.
// KBC collision (an extension of the library, no reference counterpart):
// f - feq = ds + dh, ds_i = 4.5 w_i (c_i . D . c_i) with D the deviatoric
// non-equilibrium stress, ds relaxed at omega and dh at gamma omega / 2,
// gamma = 1/beta - (2 - 1/beta) <ds|dh>/<dh|dh> (beta = omega/2, <x|y> =
// sum x_i y_i / feq_i, raw feq; 2 when <dh|dh> = 0; kept in [0, 2/beta]).
// Where F != 0 the part
// dk_i = -1.5 w_i (c_i . F) of f - feq relaxes at omega, outside dh, and the
// Guo source (1 - omega/2) w_i (3 c.F + 9 (c.u)(c.F) - 3 u.F) is added. Same
// operation order as relax_kbc in lbm_cell.cuh.
template <class R>
void relax_kbc(R* fh, R w, R rho, R rhom1, R ux, R uy, R uz, R u2, const R F[3], bool force) {
    auto geq = [&](int i) {
        const R cu = i == 0 ? R(0) : R(3) * cdot<R>(i, ux, uy, uz);
        return weight<R>(i) * (rhom1 + rho * (cu + R(0.5) * cu * cu - R(1.5) * u2));
    };
    R P[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};  // xx, yy, zz, xy, xz, yz
    bool st[6] = {false, false, false, false, false, false};
    auto acc = [&](int k, int coef, R d) {
        if (coef == 0) return;
        const R t = coef > 0 ? d : -d;
        P[k] = st[k] ? P[k] + t : t;
        st[k] = true;
    };
    for (int i = 1; i < 19; ++i) {
        const R d = fh[i] - geq(i);
        acc(0, CX[i] * CX[i], d);
        acc(1, CY[i] * CY[i], d);
        acc(2, CZ[i] * CZ[i], d);
        acc(3, CX[i] * CY[i], d);
        acc(4, CX[i] * CZ[i], d);
        acc(5, CY[i] * CZ[i], d);
    }
    const R tr = (P[0] + P[1] + P[2]) * (R(1) / R(3));
    const R dxx = P[0] - tr, dyy = P[1] - tr, dzz = P[2] - tr;
    auto cdc = [&](int i) {  // c_i . D . c_i
        const int a = CX[i], b = CY[i], c = CZ[i];
        if (i == 0) return R(0);
        if (a != 0 && b != 0) return (dxx + dyy) + R(2) * (a * b > 0 ? P[3] : -P[3]);
        if (a != 0 && c != 0) return (dxx + dzz) + R(2) * (a * c > 0 ? P[4] : -P[4]);
        if (b != 0 && c != 0) return (dyy + dzz) + R(2) * (b * c > 0 ? P[5] : -P[5]);
        return a != 0 ? dxx : (b != 0 ? dyy : dzz);
    };
    auto dk_of = [&](int i) {
        return i == 0 ? R(0) : (R(-1.5) * weight<R>(i)) * cdot<R>(i, F[0], F[1], F[2]);
    };
    auto dh_of = [&](int i, R g, R ds) {
        R dh = (fh[i] - g) - ds;
        if (force) dh = dh - dk_of(i);
        return dh;
    };
    R sh = R(0), hh = R(0);
    for (int i = 0; i < 19; ++i) {
        const R g = geq(i);
        const R ds = (R(4.5) * weight<R>(i)) * cdc(i);
        const R dh = dh_of(i, g, ds);
        const R r = dh / (g + weight<R>(i));
        sh = sh + ds * r;
        hh = hh + dh * r;
    }
    const R beta = R(0.5) * w;
    const R ib = R(1) / beta;
    const R gamma = Fmin(Fmax(hh > R(0) ? ib - (R(2) - ib) * sh / hh : R(2), R(0)), R(2) * ib);
    const R a = R(1) - R(0.5) * w;
    const R uF = ux * F[0] + uy * F[1] + uz * F[2];
    R out[19];
    for (int i = 0; i < 19; ++i) {
        const R g = geq(i);
        const R ds = (R(4.5) * weight<R>(i)) * cdc(i);
        const R dh = dh_of(i, g, ds);
        R v;
        if (force) {
            const R cF = i == 0 ? R(0) : cdot<R>(i, F[0], F[1], F[2]);
            const R cu = i == 0 ? R(0) : cdot<R>(i, ux, uy, uz);
            const R dk = (R(-1.5) * weight<R>(i)) * cF;
            v = fh[i] - beta * (R(2) * (ds + dk) + gamma * dh);
            v = v + a * weight<R>(i) * (R(3) * cF + R(9) * cu * cF - R(3) * uF);
        } else {
            v = fh[i] - beta * (R(2) * ds + gamma * dh);
        }
        out[i] = v;
    }
    for (int i = 0; i < 19; ++i) fh[i] = out[i];
}

template <class R>
void relax_fused(R* fh, R wp, R wm, R rho, R rhom1, R ux, R uy, R uz, R u2, const R F[3], R eps,
                 R nt[3]) {
    const R u2t = R(1.5) * u2;
    const R w0 = weight<R>(0), ws = weight<R>(1), wl = weight<R>(7);
    const R wr0 = w0 * rho, wm0 = w0 * rhom1;
    const R wrs = ws * rho, wms = ws * rhom1;
    const R wrl = wl * rho, wml = wl * rhom1;
    const R feq0 = Fma(-wr0, u2t, wm0);
    const R uF = Fma(uz, F[2], Fma(uy, F[1], ux * F[0]));
    const R ap = Fma(R(-0.5), wp, R(1));
    const R am = Fma(R(-0.5), wm, R(1));
    const R aps = ws * ap, apl = wl * ap, ams = ws * am, aml = wl * am;
    const R s0 = w0 * ap * (R(-3) * uF);
    const bool nt_cell = !(eps == R(0));
    R B = R(0), omb = R(1);
    if (!nt_cell) {
        fh[0] = Fma(wp, feq0 - fh[0], fh[0]) + s0;
    } else {
        const R tw = R(1) / wp - R(0.5);
        B = eps * tw / ((R(1) - eps) + tw);
        omb = R(1) - B;
        fh[0] = Fma(omb, Fma(wp, feq0 - fh[0], s0), fh[0]);
    }
    for (int i = 1; i < 19; i += 2) {
        const bool lng = i >= 7;
        const R wr = lng ? wrl : wrs, wmr = lng ? wml : wms;
        const R cd = cdot<R>(i, ux, uy, uz);
        const R X = Fma(R(4.5) * cd, cd, -u2t);
        const R feqp = Fma(wr, X, wmr);
        const R feqm = wr * (R(3) * cd);
        const R A = Fma(R(-0.5), fh[i] + fh[i + 1], feqp);
        const R Bm = Fma(R(-0.5), fh[i] - fh[i + 1], feqm);
        const R cF = cdot<R>(i, F[0], F[1], F[2]);
        const R sm = (lng ? aml : ams) * (R(3) * cF);
        const R sp = (lng ? apl : aps) * (R(3) * Fma(R(3) * cd, cF, -uF));
        const R spp = sp + sm, spm = sp - sm;
        if (!nt_cell) {
            fh[i] = Fma(wp, A, Fma(wm, Bm, fh[i] + spp));
            fh[i + 1] = Fma(wp, A, Fma(-wm, Bm, fh[i + 1] + spm));
        } else {
            const R up = Fma(wp, A, Fma(wm, Bm, spp));
            const R um = Fma(wp, A, Fma(-wm, Bm, spm));
            const R bounce = B * (fh[i + 1] - fh[i]);
            fh[i] = Fma(omb, up, bounce) + fh[i];
            fh[i + 1] = Fma(omb, um, -bounce) + fh[i + 1];
            const int c[3] = {CX[i], CY[i], CZ[i]};
            for (int k = 0; k < 3; ++k)
                if (c[k] != 0) nt[k] -= R(2 * c[k]) * bounce;
        }
    }
}

template <class R, class S> struct Field {
    S* f;
    size_t N;
    R ld(int i, size_t n) const { return R(f[size_t(i) * N + n]); }
    void st(int i, size_t n, R v) const { f[size_t(i) * N + n] = S(v); }
};

template <class R> inline void cell_force(const Params& p, const float* ffield, size_t N,
                                          size_t n, R F[3]) {
    F[0] = R(p.fx);
    F[1] = R(p.fy);
    F[2] = R(p.fz);
    if (ffield) {  // per-cell Guo force field extension: F = uniform + field[n]
        F[0] = R(p.fx + ffield[n]);
        F[1] = R(p.fy + ffield[N + n]);
        F[2] = R(p.fz + ffield[2 * N + n]);
    }
}

// Slots one cell reads and writes in one pass of the AA pattern
// (Kernels.metal:252-350): value fh_i comes from rd[i] and the post-collision
// value of direction i goes to wr[i]. In both passes the two sets coincide,
// which is what makes the update in place.
struct CellSlots {
    size_t rd[19];
    size_t wr[19];
};

inline void cell_slots(const Params& p, uint32_t sMask, size_t N, size_t n, int x, int y, int z,
                       CellSlots& c) {
    const int nx = int(p.nx), ny = int(p.ny), nz = int(p.nz);
    c.rd[0] = c.wr[0] = n;
    for (int i = 1; i < 19; ++i) {
        if (p.parity == 0u) {
            c.rd[i] = size_t(i) * N + n;
            c.wr[i] = size_t(OPP[i]) * N + n;
            continue;
        }
        if ((sMask >> (OPP[i] - 1)) & 1u) {
            c.rd[i] = size_t(i) * N + n;
        } else {
            const int sx = wrap(x - CX[i], nx), sy = wrap(y - CY[i], ny), sz = wrap(z - CZ[i], nz);
            c.rd[i] = size_t(OPP[i]) * N + (size_t(sz) * ny + sy) * nx + sx;
        }
        if ((sMask >> (i - 1)) & 1u) {
            c.wr[i] = size_t(OPP[i]) * N + n;
        } else {
            const int dx = wrap(x + CX[i], nx), dy = wrap(y + CY[i], ny), dz = wrap(z + CZ[i], nz);
            c.wr[i] = size_t(i) * N + (size_t(dz) * ny + dy) * nx + dx;
        }
    }
}

// Local update of one fluid cell from the 19 values it read (in[i] from slot
// rd[i]): out[i] is stored to slot wr[i]; a[] receives the cell's
// momentum-exchange force and force_out tells whether the reference writes it
// (Kernels.metal:240-354, same order of operations).
//
// opts: OPT_PRESSURE_OUTFLOW, OPT_KBC (library extensions, below).
// With OPT_PRESSURE_OUTFLOW (pressure outflow, an extension of the reference's dormant
// outflow wall): each link reflected from an outflow wall also gains
// w_i (9 (c_i . u)^2 - 3 u^2), u = p / rho (no force term) of the gathered
// DDFs (reflections without the terms) on the load side, before the
// collision, and of the post-collision DDFs on the store side.
template <class R, bool FUSED = false>
void cell_compute(const Params& p, const uint8_t* flags, uint32_t sMask, uint32_t lMask, int x,
                  int y, int z, const R in[19], R eps, const R F[3], R out[19], R a[3],
                  bool& force_out, int opts = 0) {
    const bool abbp = (opts & OPT_PRESSURE_OUTFLOW) != 0;
    const bool kbc = (opts & OPT_KBC) != 0;
    const int nx = int(p.nx), ny = int(p.ny), nz = int(p.nz);
    R fh[19];
    for (int i = 0; i < 19; ++i) fh[i] = in[i];
    R rho = R(1);
    R nt[3] = {R(0), R(0), R(0)};
    a[0] = a[1] = a[2] = R(0);
    force_out = false;
    if (p.parity == 0u) {  // even: in-cell pass
        collide<R, FUSED>(fh, p, x, eps, F, rho, nt, kbc);
        for (int i = 0; i < 19; ++i) out[i] = fh[i];
        if (p.writeForce != 0u && eps > R(0)) {
            a[0] = nt[0]; a[1] = nt[1]; a[2] = nt[2];
            force_out = true;
        }
        return;
    }
    // odd: streaming pass with walls
    auto acc_sub = [&](int i, R v) {  // a -= c_i * v
        const int c[3] = {CX[i], CY[i], CZ[i]};
        for (int k = 0; k < 3; ++k)
            if (c[k] != 0) a[k] = c[k] > 0 ? a[k] - v : a[k] + v;
    };
    auto acc_add = [&](int i, R v) {  // a += c_i * v
        const int c[3] = {CX[i], CY[i], CZ[i]};
        for (int k = 0; k < 3; ++k)
            if (c[k] != 0) a[k] = c[k] > 0 ? a[k] + v : a[k] - v;
    };
    uint32_t deferred = 0;
    for (int i = 1; i < 19; ++i) {
        const int srcBit = OPP[i] - 1;
        if ((sMask >> srcBit) & 1u) {
            if ((lMask >> srcBit) & 1u) deferred |= (1u << i);
            if (p.writeForce != 0u) acc_sub(i, fh[i]);
        }
    }
    uint32_t abb = 0;
    R wu[3] = {R(0), R(0), R(0)}, wu2 = R(0);
    auto abb_term = [&](int i) {
        const R cu = cdot<R>(i, wu[0], wu[1], wu[2]);
        return weight<R>(i) * (R(9) * cu * cu - R(3) * wu2);
    };
    auto estimate = [&]() {  // u = p / rho of fh, the moments' summation order
        R rhom1 = fh[0];
        for (int i = 1; i < 19; ++i) rhom1 += fh[i];
        R pc[3] = {R(0), R(0), R(0)};
        bool started[3] = {false, false, false};
        for (int i = 1; i < 19; ++i) {
            const int c[3] = {CX[i], CY[i], CZ[i]};
            for (int k = 0; k < 3; ++k) {
                if (c[k] == 0) continue;
                const R t = c[k] > 0 ? fh[i] : -fh[i];
                pc[k] = started[k] ? pc[k] + t : t;
                started[k] = true;
            }
        }
        const R inv = R(1) / (R(1) + rhom1);
        for (int k = 0; k < 3; ++k) wu[k] = pc[k] * inv;
        wu2 = wu[0] * wu[0] + wu[1] * wu[1] + wu[2] * wu[2];
    };
    if (deferred != 0u) {
        for (int i = 1; i < 19; ++i) {
            if (!((deferred >> i) & 1u)) continue;
            const int sy = wrap(y - CY[i], ny);
            const size_t s = (size_t(wrap(z - CZ[i], nz)) * ny + sy) * nx + wrap(x - CX[i], nx);
            const uint8_t wf = flags[s];
            if (wf == OUTFLOW) {
                fh[i] = -fh[i];
                abb |= 1u << i;
            } else {
                const V3<R> uw = wall_velocity<R>(wf, sy, p);
                const R cu = cdot<R>(i, uw.x, uw.y, uw.z);
                const R corr = R(6) * weight<R>(i) * cu;
                fh[i] += corr;
                if (p.writeForce != 0u) acc_sub(i, corr);
            }
        }
    }
    if (abbp && lMask != 0u) {
        estimate();
        for (int i = 1; i < 19; ++i)
            if ((abb >> i) & 1u) fh[i] += abb_term(i);
    }
    collide<R, FUSED>(fh, p, x, eps, F, rho, nt, kbc);
    a[0] += nt[0];
    a[1] += nt[1];
    a[2] += nt[2];
    if (abbp && lMask != 0u) estimate();
    out[0] = fh[0];
    for (int i = 1; i < 19; ++i) {
        const int dstBit = i - 1;
        if ((sMask >> dstBit) & 1u) {
            R corr = R(0);
            R sign = R(1);
            bool has_corr = false;
            if ((lMask >> dstBit) & 1u) {
                const int dy = wrap(y + CY[i], ny);
                const size_t d =
                    (size_t(wrap(z + CZ[i], nz)) * ny + dy) * nx + wrap(x + CX[i], nx);
                const uint8_t wf = flags[d];
                if (wf == OUTFLOW) {
                    sign = R(-1);
                } else {
                    const V3<R> uw = wall_velocity<R>(wf, dy, p);
                    corr = R(6) * weight<R>(i) * cdot<R>(i, uw.x, uw.y, uw.z);
                    has_corr = true;
                }
            }
            const R sv = sign * fh[i];
            out[i] = has_corr ? sv - corr : (abbp && sign < R(0) ? sv + abb_term(i) : sv);
            if (p.writeForce != 0u) acc_add(i, sv + R(2) * weight<R>(i));
        } else {
            out[i] = fh[i];
        }
    }
    force_out = p.writeForce != 0u && (sMask != 0u || eps > R(0));
}

// One thread of the `step` kernel, Kernels.metal:230-355. FOut is float for
// the FP32-arithmetic instances and double for the FP64 oracle.
template <class R, class S, class FOut, bool FUSED>
void step_cell(const Field<R, S>& A, const uint8_t* flags, const uint32_t* sMaskBuf,
               const uint32_t* lMaskBuf, const Params& p, FOut* force, const float* epsBuf,
               const float* ffield, size_t n, int opts) {
    const size_t N = A.N;
    if (flags && flags[n] != FLUID) return;
    const R eps = (p.useEps != 0u && epsBuf) ? R(epsBuf[n]) : R(0);
    const int x = int(n % p.nx);
    const int t = int(n / p.nx);
    const int y = t % int(p.ny);
    const int z = t / int(p.ny);
    R F[3];
    cell_force<R>(p, ffield, N, n, F);
    const uint32_t sMask = (p.parity != 0u && sMaskBuf) ? sMaskBuf[n] : 0u;
    const uint32_t lMask = (p.parity != 0u && lMaskBuf) ? lMaskBuf[n] : 0u;
    CellSlots c;
    cell_slots(p, sMask, N, n, x, y, z, c);
    R in[19], out[19], a[3];
    for (int i = 0; i < 19; ++i) in[i] = R(A.f[c.rd[i]]);
    bool fo = false;
    cell_compute<R, FUSED>(p, flags, sMask, lMask, x, y, z, in, eps, F, out, a, fo, opts);
    for (int i = 0; i < 19; ++i) A.f[c.wr[i]] = S(out[i]);
    if (fo && force) {
        force[4 * n + 0] = FOut(a[0]);
        force[4 * n + 1] = FOut(a[1]);
        force[4 * n + 2] = FOut(a[2]);
        force[4 * n + 3] = FOut(0);
    }
}

template <class R, class S, class FOut, bool FUSED = false>
void step_all(void* f, const uint8_t* flags, const uint32_t* sm, const uint32_t* lm,
              const Params& p, FOut* force, const float* eps, const float* ffield, int threads,
              int opts = 0) {
    const size_t N = size_t(p.nx) * p.ny * p.nz;
    Field<R, S> A{static_cast<S*>(f), N};
    // The AA pattern gives every slot one reader and one writer, and they are the
    // same thread, so cells may be processed in any order or in parallel.
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1) if (threads > 1)
    for (long long n = 0; n < (long long)N; ++n)
        step_cell<R, S, FOut, FUSED>(A, flags, sm, lm, p, force, eps, ffield, size_t(n), opts);
}

// momentsEven, Kernels.metal:359-380 (division by rho, not by a reciprocal).
template <class R, class S>
void moments_all(const void* fv, const uint8_t* flags, const Params& p, const float* ffield,
                 R* out) {
    const size_t N = size_t(p.nx) * p.ny * p.nz;
    const S* f = static_cast<const S*>(fv);
    for (size_t n = 0; n < N; ++n) {
        if (flags && flags[n] != FLUID) {
            out[4 * n] = out[4 * n + 1] = out[4 * n + 2] = out[4 * n + 3] = R(0);
            continue;
        }
        R v[19];
        for (int i = 0; i < 19; ++i) v[i] = R(f[size_t(i) * N + n]);
        R rhom1 = v[0];
        for (int i = 1; i < 19; ++i) rhom1 += v[i];
        R pc[3] = {0, 0, 0};
        bool st[3] = {false, false, false};
        for (int i = 1; i < 19; ++i) {
            const int c[3] = {CX[i], CY[i], CZ[i]};
            for (int k = 0; k < 3; ++k) {
                if (c[k] == 0) continue;
                const R t = c[k] > 0 ? v[i] : -v[i];
                pc[k] = st[k] ? pc[k] + t : t;
                st[k] = true;
            }
        }
        R F[3];
        cell_force<R>(p, ffield, N, n, F);
        const R rho = R(1) + rhom1;
        out[4 * n + 0] = (pc[0] + R(0.5) * F[0]) / rho;
        out[4 * n + 1] = (pc[1] + R(0.5) * F[1]) / rho;
        out[4 * n + 2] = (pc[2] + R(0.5) * F[2]) / rho;
        out[4 * n + 3] = rho;
    }
}

// Kinetic-energy and dissipation sums of a state, the library's observables
// reduction restated: per fluid cell |u|^2 (u with the half-force shift, as
// momentsEven) and 2 nu S:S with S = -(1.5 omega / rho) Pi_neq, Pi_neq the
// second moment of f - feq (full equilibrium), nu = (1/omega - 1/2)/3. R is
// the arithmetic of the per-cell values; both sums are accumulated in double,
// per thread over a static range of cells and then in thread order.
// |u|^2 (u2) and sc^2 Pi:Pi of one fluid cell from its 19 DDFs v (natural
// slots, even step count) and its Guo force F: Pi is the non-equilibrium
// second moment and sc = 1.5 omega / rho, so the cell's dissipation 2 nu S:S
// is 2 nu times the result. Shared by the observables and, in dual numbers,
// by the adjoint of the time-averaged dissipation.
template <class R>
inline R cell_strain2(const R (&v)[19], const R (&F)[3], R om, R& u2) {
    R rhom1 = v[0];
    for (int i = 1; i < 19; ++i) rhom1 += v[i];
    R pc[3] = {R(0), R(0), R(0)};
    for (int i = 1; i < 19; ++i) {
        pc[0] += R(CX[i]) * v[i];
        pc[1] += R(CY[i]) * v[i];
        pc[2] += R(CZ[i]) * v[i];
    }
    const R rho = R(1) + rhom1;
    const R ux = (pc[0] + R(0.5) * F[0]) / rho, uy = (pc[1] + R(0.5) * F[1]) / rho,
            uz = (pc[2] + R(0.5) * F[2]) / rho;
    u2 = ux * ux + uy * uy + uz * uz;
    R P[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    for (int i = 1; i < 19; ++i) {
        const R cu = R(3) * (R(CX[i]) * ux + R(CY[i]) * uy + R(CZ[i]) * uz);
        const R feq = weight<R>(i) * (rhom1 + rho * (cu + R(0.5) * cu * cu - R(1.5) * u2));
        const R d = v[i] - feq;
        P[0] += R(CX[i] * CX[i]) * d;
        P[1] += R(CY[i] * CY[i]) * d;
        P[2] += R(CZ[i] * CZ[i]) * d;
        P[3] += R(CX[i] * CY[i]) * d;
        P[4] += R(CX[i] * CZ[i]) * d;
        P[5] += R(CY[i] * CZ[i]) * d;
    }
    const R pipi = P[0] * P[0] + P[1] * P[1] + P[2] * P[2] +
                   R(2) * (P[3] * P[3] + P[4] * P[4] + P[5] * P[5]);
    const R sc = R(1.5) * om / rho;
    return sc * sc * pipi;
}

template <class R, class S>
void observables_all(const void* fv, const uint8_t* flags, const Params& p, const float* ffield,
                     double omega, int threads, double out[2]) {
    const size_t N = size_t(p.nx) * p.ny * p.nz;
    const S* f = static_cast<const S*>(fv);
    const double nu = (1.0 / omega - 0.5) / 3.0;
    const R om = R(omega);
    const int T = threads > 0 ? threads : 1;
    std::vector<double> part(2 * size_t(T), 0.0);
#pragma omp parallel num_threads(T) if (T > 1)
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        const size_t lo = N * size_t(tid) / size_t(nt), hi = N * size_t(tid + 1) / size_t(nt);
        double ke = 0.0, ds = 0.0;
        for (size_t n = lo; n < hi; ++n) {
            if (flags && flags[n] != FLUID) continue;
            R v[19];
            for (int i = 0; i < 19; ++i) v[i] = R(f[size_t(i) * N + n]);
            R F[3];
            cell_force<R>(p, ffield, N, n, F);
            R u2;
            const R t = cell_strain2<R>(v, F, om, u2);
            ke += double(u2);
            ds += 2.0 * nu * double(t);
        }
        part[2 * size_t(tid)] = ke;
        part[2 * size_t(tid) + 1] = ds;
    }
    out[0] = out[1] = 0.0;
    for (int t = 0; t < T; ++t) {
        out[0] += part[2 * size_t(t)];
        out[1] += part[2 * size_t(t) + 1];
    }
}

// initField, Kernels.metal:393-453. Trigonometric values are evaluated in
// double and rounded to R, so FP32 results are the correctly rounded sin/cos.
template <class R> inline R tsin(R a) { return R(std::sin(double(a))); }
template <class R> inline R tcos(R a) { return R(std::cos(double(a))); }

template <class R, class S>
void init_all(void* fv, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t mode, float amplitude,
              float tau) {
    const size_t N = size_t(nx) * ny * nz;
    S* f = static_cast<S*>(fv);
    const R A = R(amplitude);
    const R pi = sizeof(R) == 4 ? R(3.14159265358979323846f) : R(3.14159265358979323846);
    for (size_t n = 0; n < N; ++n) {
        R ux = 0, uy = 0, uz = 0, sxx = 0, sxz = 0, syz = 0, rhom1 = 0;
        const uint32_t x = uint32_t(n % nx), t = uint32_t(n / nx), y = t % ny, z = t / ny;
        if (mode == 1u) {
            const R kx = R(2) * pi / R(nx), ky = R(2) * pi / R(ny);
            const R xa = R(x) + R(0.5), ya = R(y) + R(0.5);
            ux = A * tsin(kx * xa) * tcos(ky * ya);
            uy = -A * tcos(kx * xa) * tsin(ky * ya);
            sxx = A * kx * tcos(kx * xa) * tcos(ky * ya);
            rhom1 = R(0.75) * A * A * (tcos(R(2) * kx * xa) + tcos(R(2) * ky * ya));
        }
        if (mode == 2u) {
            const R kx = R(2) * pi / R(nx), ky = R(2) * pi / R(ny), kz = R(2) * pi / R(nz);
            const R xa = kx * (R(x) + R(0.5)), ya = ky * (R(y) + R(0.5)), za = kz * (R(z) + R(0.5));
            ux = A * tsin(xa) * tcos(ya) * tcos(za);
            uy = -A * tcos(xa) * tsin(ya) * tcos(za);
            sxx = A * kx * tcos(xa) * tcos(ya) * tcos(za);
            sxz = R(-0.5) * A * kz * tsin(xa) * tcos(ya) * tsin(za);
            syz = R(0.5) * A * kz * tcos(xa) * tsin(ya) * tsin(za);
            rhom1 = R(0.1875) * A * A * (tcos(R(2) * xa) + tcos(R(2) * ya)) * (tcos(R(2) * za) + R(2));
        }
        const R rho = R(1) + rhom1;
        const R u2 = ux * ux + uy * uy + uz * uz;
        for (int i = 0; i < 19; ++i) {
            const R cu = R(3) * (R(CX[i]) * ux + R(CY[i]) * uy + R(CZ[i]) * uz);
            const R feq = weight<R>(i) * (rhom1 + rho * (cu + R(0.5) * cu * cu - R(1.5) * u2));
            const R cc = R(CX[i] * CX[i] - CY[i] * CY[i]);
            const R scc = sxx * cc + R(2) * sxz * R(CX[i] * CZ[i]) + R(2) * syz * R(CY[i] * CZ[i]);
            const R fneq = R(-3) * weight<R>(i) * R(tau) * scc;
            f[size_t(i) * N + n] = S(feq + fneq);
        }
    }
}

}  // namespace

// Forward and reverse steps of the FP64 adjoint (orc_adjoint_force_ex below).
namespace adj {

struct Ctx {
    const uint8_t* flags;
    const uint32_t* solid_mask;
    const uint32_t* lid_mask;
    const float* eps;
    const float* ffield;
    const int* box;
    const double* dir;
    size_t N;
    int threads;
};

inline void cell_ctx(const Params& p, const Ctx& c, size_t n, int& x, int& y, int& z,
                     uint32_t& sm, uint32_t& lm) {
    x = int(n % p.nx);
    const int t = int(n / p.nx);
    y = t % int(p.ny);
    z = t / int(p.ny);
    sm = (p.parity != 0u && c.solid_mask) ? c.solid_mask[n] : 0u;
    lm = (p.parity != 0u && c.lid_mask) ? c.lid_mask[n] : 0u;
}

inline bool in_box(const Ctx& c, int x, int y) {
    return x >= c.box[0] && x <= c.box[1] && y >= c.box[2] && y <= c.box[3];
}

// One forward step of A in place in arithmetic R, each stored value rounded to
// S; contrib[n] = dir . a of the cells whose force counts (0 elsewhere).
template <class R, class S>
void step(const Params& p, const Ctx& c, double* A, double* contrib) {
    const long long N = (long long)c.N;
#pragma omp parallel for schedule(static) num_threads(c.threads > 0 ? c.threads : 1) if (c.threads > 1)
    for (long long nn = 0; nn < N; ++nn) {
        const size_t n = size_t(nn);
        contrib[n] = 0.0;
        if (c.flags && c.flags[n] != FLUID) continue;
        int x, y, z;
        uint32_t sm, lm;
        cell_ctx(p, c, n, x, y, z, sm, lm);
        CellSlots cs;
        cell_slots(p, sm, c.N, n, x, y, z, cs);
        R in[19], out[19], a[3], F[3];
        for (int i = 0; i < 19; ++i) in[i] = R(A[cs.rd[i]]);
        cell_force<R>(p, c.ffield, c.N, n, F);
        const R e = (p.useEps && c.eps) ? R(c.eps[n]) : R(0);
        bool fo = false;
        cell_compute<R>(p, c.flags, sm, lm, x, y, z, in, e, F, out, a, fo);
        for (int i = 0; i < 19; ++i) A[cs.wr[i]] = double(S(out[i]));
        if (p.parity && fo && in_box(c, x, y))
            contrib[n] = c.dir[0] * double(a[0]) + c.dir[1] * double(a[1]) +
                         c.dir[2] * double(a[2]);
    }
}

inline void step_traj(int traj, const Params& p, const Ctx& c, double* A, double* contrib) {
    if (traj == 0) step<float, float>(p, c, A, contrib);
    else if (traj == 1) step<float, _Float16>(p, c, A, contrib);
    else step<double, double>(p, c, A, contrib);
}

// Reverse of one step about its input state S: lam (the adjoint of the state
// after the step) becomes the adjoint of the state before it; the parameter
// adjoints are accumulated.
void reverse(const Params& p, const Ctx& c, const double* S, double* lam, double w,
             double* grad_eps, double* grad_f) {
    typedef Dual<23> D;
    const long long N = (long long)c.N;
#pragma omp parallel for schedule(static) num_threads(c.threads > 0 ? c.threads : 1) if (c.threads > 1)
    for (long long nn = 0; nn < N; ++nn) {
        const size_t n = size_t(nn);
        if (c.flags && c.flags[n] != FLUID) continue;
        int x, y, z;
        uint32_t sm, lm;
        cell_ctx(p, c, n, x, y, z, sm, lm);
        CellSlots cs;
        cell_slots(p, sm, c.N, n, x, y, z, cs);
        D in[19], out[19], a[3], F[3];
        for (int i = 0; i < 19; ++i) in[i] = D::var(S[cs.rd[i]], i);
        double Fv[3];
        cell_force<double>(p, c.ffield, c.N, n, Fv);
        for (int k = 0; k < 3; ++k) F[k] = D::var(Fv[k], 20 + k);
        const D e = D::var((p.useEps && c.eps) ? double(c.eps[n]) : 0.0, 19);
        bool fo = false;
        cell_compute<D>(p, c.flags, sm, lm, x, y, z, in, e, F, out, a, fo);
        double mu[19];
        for (int j = 0; j < 19; ++j) mu[j] = lam[cs.wr[j]];
        const bool obj = p.parity && fo && in_box(c, x, y);
        double g[23];
        for (int k = 0; k < 23; ++k) {
            double acc = 0.0;
            for (int j = 0; j < 19; ++j) acc += mu[j] * out[j].d[k];
            if (obj)
                acc += w * (c.dir[0] * a[0].d[k] + c.dir[1] * a[1].d[k] + c.dir[2] * a[2].d[k]);
            g[k] = acc;
        }
        for (int i = 0; i < 19; ++i) lam[cs.rd[i]] = g[i];
        if (grad_eps) grad_eps[n] += g[19];
        if (grad_f)
            for (int k = 0; k < 3; ++k) grad_f[k * c.N + n] += g[20 + k];
    }
}

// Sum of 2 nu S:S over the fluid cells of the state A (an even step count),
// in FP64: the dissipation observable of the adjoint's dissipation objective.
double dissipation(const Params& p, const Ctx& c, const double* A, double omega) {
    const double nu = (1.0 / omega - 0.5) / 3.0;
    double out = 0.0;
    for (size_t n = 0; n < c.N; ++n) {
        if (c.flags && c.flags[n] != FLUID) continue;
        double v[19], F[3], u2;
        for (int i = 0; i < 19; ++i) v[i] = A[size_t(i) * c.N + n];
        cell_force<double>(p, c.ffield, c.N, n, F);
        out += 2.0 * nu * cell_strain2<double>(v, F, omega, u2);
    }
    return out;
}

// lam += w dD/dA and grad_f += w dD/dF_field for the dissipation D of the
// state A (natural slots at an even step count), each cell's gradient from
// dual numbers over its 19 DDFs and its force.
void inject_dissipation(const Params& p, const Ctx& c, const double* A, double omega, double w,
                        double* lam, double* grad_f) {
    typedef Dual<22> D;
    const double nu = (1.0 / omega - 0.5) / 3.0;
    const long long N = (long long)c.N;
#pragma omp parallel for schedule(static) num_threads(c.threads > 0 ? c.threads : 1) if (c.threads > 1)
    for (long long nn = 0; nn < N; ++nn) {
        const size_t n = size_t(nn);
        if (c.flags && c.flags[n] != FLUID) continue;
        D v[19], F[3], u2;
        for (int i = 0; i < 19; ++i) v[i] = D::var(A[size_t(i) * c.N + n], i);
        double Fv[3];
        cell_force<double>(p, c.ffield, c.N, n, Fv);
        for (int k = 0; k < 3; ++k) F[k] = D::var(Fv[k], 19 + k);
        const D t = cell_strain2<D>(v, F, D(omega), u2);
        const double g = w * 2.0 * nu;
        for (int i = 0; i < 19; ++i) lam[size_t(i) * c.N + n] += g * t.d[i];
        if (grad_f)
            for (int k = 0; k < 3; ++k) grad_f[size_t(k) * c.N + n] += g * t.d[19 + k];
    }
}

}  // namespace adj

extern "C" {

// kind: 0 = <float,float>, 1 = <float,_Float16>, 2 = <double,double>;
// orc_step also takes 3 = <float,float> and 4 = <float,_Float16> in the fused
// arithmetic.

// Neighbour masks, Sim.swift:227-255: bit i-1 of solid_mask is set when the
// neighbour at n + c_i is not fluid; lid_mask marks the moving-wall subset.
int orc_masks(const uint8_t* flags, int nx, int ny, int nz, uint32_t* solid_mask,
              uint32_t* lid_mask) {
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const size_t idx = (size_t(z) * ny + y) * nx + x;
                uint32_t s = 0, l = 0;
                if (flags[idx] == FLUID) {
                    for (int i = 1; i < 19; ++i) {
                        const int xn = (x + CX[i] + nx) % nx, yn = (y + CY[i] + ny) % ny,
                                  zn = (z + CZ[i] + nz) % nz;
                        const uint8_t c = flags[(size_t(zn) * ny + yn) * nx + xn];
                        if (c == FLUID) continue;
                        s |= 1u << (i - 1);
                        if (c == LID || c == INFLOW || c == OUTFLOW) l |= 1u << (i - 1);
                    }
                }
                solid_mask[idx] = s;
                lid_mask[idx] = l;
            }
    return 0;
}

// Per-step uniforms with the C1 cosine ramp, Sim.swift:258-281. sponge_width
// <= 0 disables the sponge (x0 = 1e9, 1/w = 0, tau = 1).
int orc_params(void* out, uint32_t nx, uint32_t ny, uint32_t nz, long long step, float omega,
               float omega_minus, float uin_target, long long ramp_steps, float cSmago,
               const float force[3], int write_force, const float lid[3], int inflow_uniform,
               float sponge_x0, float sponge_width, float sponge_tau, int use_eps) {
    Params p{};
    float r = 1.0f;
    if (ramp_steps > 0) {
        const double x = std::fmin(1.0, double(step) / double(ramp_steps));
        r = 1.0f * float(0.5 * (1.0 - std::cos(3.141592653589793 * x)));
    }
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.parity = uint32_t(step & 1);
    p.omega = omega; p.omegaMinus = omega_minus;
    p.uin = uin_target * r;
    p.cSmago = cSmago;
    p.fx = force[0]; p.fy = force[1]; p.fz = force[2];
    p.writeForce = write_force ? 1u : 0u;
    p.ulidX = lid[0] * r; p.ulidY = lid[1] * r; p.ulidZ = lid[2] * r;
    p.inflowUniform = inflow_uniform ? 1u : 0u;
    if (sponge_width > 0.0f) {
        p.spongeX0 = sponge_x0; p.spongeInvW = 1.0f / sponge_width; p.spongeTau = sponge_tau;
    } else {
        p.spongeX0 = 1e9f; p.spongeInvW = 0.0f; p.spongeTau = 1.0f;
    }
    p.useEps = use_eps ? 1u : 0u;
    std::memcpy(out, &p, sizeof p);
    return 0;
}

// One full step over all cells. force: N*4 float (kinds 0/1) or double (kind 2),
// or null. ffield: optional per-cell force field, 3 planes of N floats.
// kind | ORC_PRESSURE_OUTFLOW: outflow walls with the pressure terms;
// kind | ORC_KBC: the KBC collision.
constexpr int ORC_PRESSURE_OUTFLOW = 0x100;
constexpr int ORC_KBC = 0x200;
int orc_step(int kind, void* f, const uint8_t* flags, const uint32_t* solid_mask,
             const uint32_t* lid_mask, const void* params, void* force, const float* eps,
             const float* ffield, int threads) {
    Params p;
    std::memcpy(&p, params, sizeof p);
    const int abbp = ((kind & ORC_PRESSURE_OUTFLOW) ? OPT_PRESSURE_OUTFLOW : 0) |
                     ((kind & ORC_KBC) ? OPT_KBC : 0);
    switch (kind & ~(ORC_PRESSURE_OUTFLOW | ORC_KBC)) {
        case 0: step_all<float, float, float>(f, flags, solid_mask, lid_mask, p,
                                              static_cast<float*>(force), eps, ffield, threads,
                                              abbp);
                return 0;
        case 1: step_all<float, _Float16, float>(f, flags, solid_mask, lid_mask, p,
                                                 static_cast<float*>(force), eps, ffield, threads,
                                                 abbp);
                return 0;
        case 2: step_all<double, double, double>(f, flags, solid_mask, lid_mask, p,
                                                 static_cast<double*>(force), eps, ffield, threads,
                                                 abbp);
                return 0;
        case 3: step_all<float, float, float, true>(f, flags, solid_mask, lid_mask, p,
                                                    static_cast<float*>(force), eps, ffield, threads,
                                                    abbp);
                return 0;
        case 4: step_all<float, _Float16, float, true>(f, flags, solid_mask, lid_mask, p,
                                                       static_cast<float*>(force), eps, ffield,
                                                       threads, abbp);
                return 0;
    }
    return 1;
}

// (ux, uy, uz, rho) per cell; out is N*4 float (kinds 0/1) or double (kind 2).
int orc_moments(int kind, const void* f, const uint8_t* flags, const void* params,
                const float* ffield, void* out) {
    Params p;
    std::memcpy(&p, params, sizeof p);
    switch (kind) {
        case 0: moments_all<float, float>(f, flags, p, ffield, static_cast<float*>(out)); return 0;
        case 1: moments_all<float, _Float16>(f, flags, p, ffield, static_cast<float*>(out)); return 0;
        case 2: moments_all<double, double>(f, flags, p, ffield, static_cast<double*>(out)); return 0;
    }
    return 1;
}

// Kinetic-energy and dissipation sums (observables_all above): out[0] = sum
// |u|^2, out[1] = sum 2 nu S:S over fluid cells; kinds 0/1/2 as orc_moments.
int orc_observables(int kind, const void* f, const uint8_t* flags, const void* params,
                    const float* ffield, double omega, int threads, double* out) {
    Params p;
    std::memcpy(&p, params, sizeof p);
    switch (kind) {
        case 0: observables_all<float, float>(f, flags, p, ffield, omega, threads, out); return 0;
        case 1: observables_all<float, _Float16>(f, flags, p, ffield, omega, threads, out); return 0;
        case 2: observables_all<double, double>(f, flags, p, ffield, omega, threads, out); return 0;
    }
    return 1;
}

int orc_init_field(int kind, void* f, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t mode,
                   float amplitude, float tau) {
    switch (kind) {
        case 0: init_all<float, float>(f, nx, ny, nz, mode, amplitude, tau); return 0;
        case 1: init_all<float, _Float16>(f, nx, ny, nz, mode, amplitude, tau); return 0;
        case 2: init_all<double, double>(f, nx, ny, nz, mode, amplitude, tau); return 0;
    }
    return 1;
}

// FP64 discrete adjoint of the time-averaged momentum-exchange force, by
// forward-mode automatic differentiation of the restated step (Dual<23>)
// for the local Jacobians and a reverse sweep over the steps.
//   J = (1/K) sum over the K odd steps t of dir . F_box(t),
// F_box(t) = sum of the per-cell force of the odd pass (the reference's force
// probe, Kernels.metal:263-353) over cells with box[0] <= x <= box[1],
// box[2] <= y <= box[3], all z. params: `steps` consecutive 80-byte Params
// (writeForce is set here on odd steps). f0: initial state, 19*N doubles.
//
// traj selects the forward trajectory the adjoint linearises about:
//   2  FP64 arithmetic and storage (the FP64 oracle);
//   0  FP32 arithmetic over FP32 storage, 1  FP32 arithmetic over FP16 storage:
//      the library's forward step value for value, so the local Jacobians are
//      taken in FP64 at exactly the stored states the GPU's reverse pass sees
//      (f0 must then hold values of the storage type).
// chk: checkpoint interval; the window's states are recomputed segment by
// segment from checkpoints (0 = one segment). threads: OpenMP threads over cells
// (the AA pattern gives every slot one reader and one writer, the same cell, in
// both the forward and the reverse step). Outputs J and, when grad_eps /
// grad_f are not null, dJ/d eps (N) and dJ/d F_field (3 planes of N); with
// both null no state is stored.

int orc_adjoint_force_ex(int traj, const double* f0, const uint8_t* flags,
                         const uint32_t* solid_mask, const uint32_t* lid_mask, const void* params,
                         int steps, const float* eps, const float* ffield, const int box[4],
                         const double dir[3], int threads, int chk, double* J_out,
                         double* grad_eps, double* grad_f) {
    if (steps <= 0 || traj < 0 || traj > 2) return 1;
    std::vector<Params> P(steps);
    std::memcpy(P.data(), params, sizeof(Params) * steps);
    const size_t N = size_t(P[0].nx) * P[0].ny * P[0].nz;
    int K = 0;
    for (int t = 0; t < steps; ++t) {
        P[t].writeForce = P[t].parity;
        K += P[t].parity ? 1 : 0;
    }
    const double w = K > 0 ? 1.0 / K : 0.0;
    const adj::Ctx c{flags, solid_mask, lid_mask, eps, ffield, box, dir, N, threads};
    const bool grads = grad_eps || grad_f;
    if (chk <= 0 || chk > steps) chk = steps;
    const int nseg = (steps + chk - 1) / chk;
    std::vector<double> A(f0, f0 + 19 * N), contrib(N);
    std::vector<std::vector<double>> ckpt(grads ? nseg : 0);
    double J = 0.0;
    for (int t = 0; t < steps; ++t) {  // forward; checkpoints at the segment starts
        if (grads && t % chk == 0) ckpt[t / chk] = A;
        adj::step_traj(traj, P[t], c, A.data(), contrib.data());
        double s = 0.0;
        for (size_t n = 0; n < N; ++n) s += contrib[n];
        J += w * s;
    }
    *J_out = J;
    if (!grads) return 0;
    if (grad_eps) std::fill(grad_eps, grad_eps + N, 0.0);
    if (grad_f) std::fill(grad_f, grad_f + 3 * N, 0.0);
    std::vector<double> lam(19 * N, 0.0);
    std::vector<std::vector<double>> seg(chk);
    for (int s = nseg - 1; s >= 0; --s) {  // reverse, one recomputed segment at a time
        const int t0 = s * chk, t1 = std::min(steps, t0 + chk);
        seg[0] = ckpt[s];
        for (int t = t0 + 1; t < t1; ++t) {
            seg[t - t0] = seg[t - t0 - 1];
            adj::step_traj(traj, P[t - 1], c, seg[t - t0].data(), contrib.data());
        }
        for (int t = t1 - 1; t >= t0; --t)
            adj::reverse(P[t], c, seg[t - t0].data(), lam.data(), w, grad_eps, grad_f);
        ckpt[s].clear();
        ckpt[s].shrink_to_fit();
    }
    return 0;
}

// FP64 discrete adjoint of the time-averaged dissipation
//   J = (1/K) sum over m = 1..K of D(t0 + m every),  K = steps / every,
// D = sum over fluid cells of 2 nu S:S of the state after m every steps of the
// window (orc_observables' out[1], evaluated in FP64 from the stored values;
// every even, the window starting at an even step count, so the sampled
// states have natural slots). traj, params, chk, threads and the outputs as
// orc_adjoint_force_ex; omega is the lattice's (nu = (1/omega - 1/2) / 3).
// D depends on the force field directly (u = (p + F/2) / rho) and through the
// dynamics; on eps only through the dynamics.
int orc_adjoint_dissipation_ex(int traj, const double* f0, const uint8_t* flags,
                               const uint32_t* solid_mask, const uint32_t* lid_mask,
                               const void* params, int steps, int every, double omega,
                               const float* eps, const float* ffield, int threads, int chk,
                               double* J_out, double* grad_eps, double* grad_f) {
    if (steps <= 0 || traj < 0 || traj > 2 || every <= 0 || every % 2 != 0) return 1;
    const int K = steps / every;
    if (K < 1) return 1;
    std::vector<Params> P(steps);
    std::memcpy(P.data(), params, sizeof(Params) * steps);
    if (P[0].parity != 0u) return 1;  // the window starts at an even step count
    for (int t = 0; t < steps; ++t) P[t].writeForce = 0u;
    const size_t N = size_t(P[0].nx) * P[0].ny * P[0].nz;
    const double w = 1.0 / K;
    const int nobox[4] = {0, -1, 0, -1};
    const double nodir[3] = {0.0, 0.0, 0.0};
    const adj::Ctx c{flags, solid_mask, lid_mask, eps, ffield, nobox, nodir, N, threads};
    const bool grads = grad_eps || grad_f;
    if (chk <= 0 || chk > steps) chk = steps;
    const int nseg = (steps + chk - 1) / chk;
    std::vector<double> A(f0, f0 + 19 * N), contrib(N);
    std::vector<std::vector<double>> ckpt(grads ? nseg : 0);
    double J = 0.0;
    for (int t = 0; t < steps; ++t) {  // forward; checkpoints at the segment starts
        if (grads && t % chk == 0) ckpt[t / chk] = A;
        adj::step_traj(traj, P[t], c, A.data(), contrib.data());
        if ((t + 1) % every == 0 && (t + 1) / every <= K)
            J += w * adj::dissipation(P[0], c, A.data(), omega);
    }
    *J_out = J;
    if (!grads) return 0;
    if (grad_eps) std::fill(grad_eps, grad_eps + N, 0.0);
    if (grad_f) std::fill(grad_f, grad_f + 3 * N, 0.0);
    std::vector<double> lam(19 * N, 0.0);
    if (steps % every == 0)  // the final state is the last sample
        adj::inject_dissipation(P[0], c, A.data(), omega, w, lam.data(), grad_f);
    std::vector<std::vector<double>> seg(chk);
    for (int s = nseg - 1; s >= 0; --s) {  // reverse, one recomputed segment at a time
        const int t0 = s * chk, t1 = std::min(steps, t0 + chk);
        seg[0] = ckpt[s];
        for (int t = t0 + 1; t < t1; ++t) {
            seg[t - t0] = seg[t - t0 - 1];
            adj::step_traj(traj, P[t - 1], c, seg[t - t0].data(), contrib.data());
        }
        for (int t = t1 - 1; t >= t0; --t) {
            adj::reverse(P[t], c, seg[t - t0].data(), lam.data(), 0.0, grad_eps, grad_f);
            // lam is now the adjoint of the state after t steps: a sample there?
            if (t > 0 && t % every == 0 && t / every <= K)
                adj::inject_dissipation(P[0], c, seg[t - t0].data(), omega, w, lam.data(),
                                        grad_f);
        }
        ckpt[s].clear();
        ckpt[s].shrink_to_fit();
    }
    return 0;
}

// The FP64 trajectory, every state kept, one thread.
int orc_adjoint_force(const double* f0, const uint8_t* flags, const uint32_t* solid_mask,
                      const uint32_t* lid_mask, const void* params, int steps, const float* eps,
                      const float* ffield, const int box[4], const double dir[3], double* J_out,
                      double* grad_eps, double* grad_f) {
    return orc_adjoint_force_ex(2, f0, flags, solid_mask, lid_mask, params, steps, eps, ffield,
                                box, dir, 1, 0, J_out, grad_eps, grad_f);
}

// Noble-Torczynski solid fractions of a closed triangle mesh by parity ray
// casting along +x, StlVoxels.swift:52-117: 2x2 sub-rays per (y, z) cell,
// exact interior x-spans, coverage accumulated per sub-ray in (sy, sz) order,
// clamped to 1. tris: ntri x 9 floats (three vertices, mesh coordinates);
// lattice coordinates are vertex * scale + offset, cell centres at integers.
// FP32 throughout, operations in the reference's order (no contraction).
// Returns 0.
int orc_mesh_solid_fractions(const float* tris, int ntri, int nx, int ny, int nz, float scale,
                             const float offset[3], float* eps) {
    struct P3 { float x, y, z; };
    std::vector<P3> t(size_t(ntri) * 3);
    for (size_t k = 0; k < t.size(); ++k) {
        t[k].x = tris[3 * k + 0] * scale + offset[0];
        t[k].y = tris[3 * k + 1] * scale + offset[1];
        t[k].z = tris[3 * k + 2] * scale + offset[2];
    }
    std::vector<std::vector<int>> buckets(size_t(ny) * nz);
    for (int i = 0; i < ntri; ++i) {
        const P3 &a = t[3 * i], &b = t[3 * i + 1], &c = t[3 * i + 2];
        const int ylo = std::max(0, int(std::floor(std::min(std::min(a.y, b.y), c.y) - 0.5f)));
        const int yhi = std::min(ny - 1, int(std::ceil(std::max(std::max(a.y, b.y), c.y) + 0.5f)));
        const int zlo = std::max(0, int(std::floor(std::min(std::min(a.z, b.z), c.z) - 0.5f)));
        const int zhi = std::min(nz - 1, int(std::ceil(std::max(std::max(a.z, b.z), c.z) + 0.5f)));
        if (ylo > yhi || zlo > zhi) continue;
        for (int z = zlo; z <= zhi; ++z)
            for (int y = ylo; y <= yhi; ++y) buckets[size_t(z) * ny + y].push_back(i);
    }
    std::fill(eps, eps + size_t(nx) * ny * nz, 0.0f);
    const int sub = 2;
    std::vector<float> xs;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const std::vector<int>& cands = buckets[size_t(z) * ny + y];
            if (cands.empty()) continue;
            for (int sy = 0; sy < sub; ++sy)
                for (int sz = 0; sz < sub; ++sz) {
                    const float ry = float(y) - 0.5f + (float(sy) + 0.5f) / float(sub);
                    const float rz = float(z) - 0.5f + (float(sz) + 0.5f) / float(sub);
                    xs.clear();
                    for (int i : cands) {
                        const P3 &a = t[3 * i], &b = t[3 * i + 1], &c = t[3 * i + 2];
                        const float d1x = b.y - a.y, d1y = b.z - a.z;
                        const float d2x = c.y - a.y, d2y = c.z - a.z;
                        const float denom = d1x * d2y - d1y * d2x;
                        if (std::fabs(denom) < 1e-12f) continue;  // ray-parallel triangle
                        const float px = ry - a.y, py = rz - a.z;
                        const float u = (px * d2y - py * d2x) / denom;
                        const float v = (d1x * py - d1y * px) / denom;
                        if (u < 0.0f || v < 0.0f || u + v > 1.0f) continue;
                        xs.push_back(a.x + u * (b.x - a.x) + v * (c.x - a.x));
                    }
                    if (xs.size() < 2) continue;
                    std::sort(xs.begin(), xs.end());
                    size_t k = 0;
                    while (k + 1 < xs.size()) {
                        if (xs[k + 1] - xs[k] < 1e-5f) {  // grazing hit
                            k += 1;
                            continue;
                        }
                        const float x0 = xs[k], x1 = xs[k + 1];
                        k += 2;
                        const int c0 = std::max(0, int(std::floor(x0 + 0.5f)));
                        const int c1 = std::min(nx - 1, int(std::floor(x1 + 0.5f)));
                        for (int x = c0; x <= c1; ++x) {
                            const float lo = float(x) - 0.5f, hi = float(x) + 0.5f;
                            const float cover = std::min(x1, hi) - std::max(x0, lo);
                            if (cover > 0.0f)
                                eps[(size_t(z) * ny + y) * nx + x] += cover / float(sub * sub);
                        }
                    }
                }
        }
    for (size_t i = 0; i < size_t(nx) * ny * nz; ++i) eps[i] = std::min(eps[i], 1.0f);
    return 0;
}

// The |u| colormap of one z slice, colorize + speedColor (Kernels.metal:465-500):
// moments4 = N float4 (momentsEven output), out = nx*ny*4 binary16 values
// (RGBA, row y written at ny-1-y). Walls and cells with eps >= 0.5 are slate;
// other cells take the four-stop map of clamp(|u| / uref, 0, 1), blended toward
// slate by eps when 0 < eps < 0.5. Vector mixes are a + (b - a) t in float; the
// half blend is evaluated in float and rounded once. Returns 0.
int orc_colorize(const float* moments4, const uint8_t* flags, const float* eps, int nx, int ny,
                 int z_slice, float uref, int use_eps, uint16_t* out) {
    typedef _Float16 h16;
    auto mix3 = [](const float* a, const float* b, float t, float* o) {
        for (int k = 0; k < 3; ++k) o[k] = a[k] + (b[k] - a[k]) * t;
    };
    const float c0[3] = {float(0.055), float(0.045), float(0.040)};
    const float c1[3] = {float(0.420), float(0.100), float(0.050)};
    const float c2[3] = {float(0.900), float(0.450), float(0.100)};
    const float c3[3] = {float(1.000), float(0.930), float(0.780)};
    const h16 slate[3] = {h16(float(0.30L)), h16(float(0.28L)), h16(float(0.25L))};
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            const size_t n = (size_t(z_slice) * ny + y) * nx + x;
            const float e = use_eps ? eps[n] : 0.0f;
            h16 rgb[3];
            if (flags[n] != FLUID || e >= 0.5f) {
                rgb[0] = slate[0]; rgb[1] = slate[1]; rgb[2] = slate[2];
            } else {
                const float* u = moments4 + 4 * n;
                const float len = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                const float s = std::fmin(std::fmax(len / uref, 0.0f), 1.0f);
                float c[3];
                if (s < 0.35f) mix3(c0, c1, s / 0.35f, c);
                else if (s < 0.70f) mix3(c1, c2, (s - 0.35f) / 0.35f, c);
                else mix3(c2, c3, (s - 0.70f) / 0.30f, c);
                for (int k = 0; k < 3; ++k) rgb[k] = h16(c[k]);
                if (e > 0.0f) {
                    const float t = float(h16(e));
                    for (int k = 0; k < 3; ++k)
                        rgb[k] = h16(float(rgb[k]) + (float(slate[k]) - float(rgb[k])) * t);
                }
            }
            const size_t o = 4 * (size_t(ny - 1 - y) * nx + x);
            const h16 px[4] = {rgb[0], rgb[1], rgb[2], h16(1.0f)};
            std::memcpy(out + o, px, sizeof px);
        }
    return 0;
}

// Sum of all 19*N shifted DDFs in index order, in double (Sim.swift:447-458).
double orc_mass(int kind, const void* f, size_t count) {
    double total = 0.0;
    for (size_t k = 0; k < count; ++k) {
        if (kind == 0) total += double(static_cast<const float*>(f)[k]);
        else if (kind == 1) total += double(static_cast<const _Float16*>(f)[k]);
        else total += static_cast<const double*>(f)[k];
    }
    return total;
}

}  // extern "C"
