// Uncertainty budget of a time-averaged quantity of interest, restating
// Sources/StrouhalCore/Uncertainty.swift with the same operation order:
//   U(phi) = k * sqrt(u_num^2 + u_stat^2 + u_Ma^2), k = 2, only inside (or
//   near the edge of) the validated domain.
// Host-only double arithmetic (compiled with -ffp-contract=off like the rest
// of the library's host code), so results are reproducible across hosts.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "strouhal_c.h"

namespace stro {
namespace rt {
int fail(int code, const std::string& msg);
}  // namespace rt
}  // namespace stro

using stro::rt::fail;

namespace {

const double kNaN = std::numeric_limits<double>::quiet_NaN();

// max(x, y) as the reference's language defines it for doubles: y when y >= x,
// else x (so a NaN first argument wins and a NaN second one loses, unlike fmax).
double smax(double x, double y) { return y >= x ? y : x; }

// Batch-means statistics with M batches (Uncertainty.swift:72-88).
void batch_stats(const double* v, int64_t n, int M, double* mean, double* half, double* rho) {
    const int64_t per = n / M;
    std::vector<double> means(static_cast<size_t>(M));
    for (int b = 0; b < M; ++b) {
        double s = 0.0;
        for (int64_t k = b * per; k < (b + 1) * per; ++k) s += v[k];
        means[size_t(b)] = s / double(per);
    }
    double m = 0.0;
    for (double x : means) m += x;
    m = m / double(M);
    double var_sum = 0.0;
    for (double x : means) var_sum = var_sum + (x - m) * (x - m);
    const double sd = std::sqrt(var_sum / double(M - 1));
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < means.size(); ++i) {
        den += (means[i] - m) * (means[i] - m);
        if (i > 0) num += (means[i] - m) * (means[i - 1] - m);
    }
    *mean = m;
    *half = 1.96 * sd / std::sqrt(double(M));
    *rho = den > 0 ? num / den : kNaN;
}

struct Anchor {
    const char* name;
    double re_lo, re_hi, ma_lo, ma_hi;
    int n_lo, n_hi;
    const char* geometry;
};

// The validated domain: the reference's anchors (Uncertainty.swift:200-213).
const Anchor kAnchors[] = {
    {"Ghia lid-driven cavity (RMS 0.004 vs published)", 100, 1000, 0, 0.18, 128, 256, "enclosed"},
    {"Sch\xc3\xa4" "fer\xe2\x80\x93Turek DFG 2D-1 (C_D within 0.16%)", 20, 20, 0, 0.14, 40, 64,
     "bluff body in channel"},
    {"Sch\xc3\xa4" "fer\xe2\x80\x93Turek DFG 2D-2 (St 0.2996, max C_L 0.9998)", 100, 100, 0, 0.14,
     40, 80, "bluff body in channel"},
    {"Poiseuille (exact) / Taylor\xe2\x80\x93Green (order 1.96)", 0, 100, 0, 0.35, 32, 128,
     "periodic / channel"},
};
const int kNumAnchors = int(sizeof(kAnchors) / sizeof(kAnchors[0]));

// Fractional distance of x outside [lo, hi], 0 inside (Uncertainty.swift:254-259).
double distance(double x, double lo, double hi) {
    if (x >= lo && x <= hi) return 0.0;
    const double span = smax(smax(hi - lo, std::fabs(hi) * 0.5), 1e-9);
    return x < lo ? (lo - x) / span : (x - hi) / span;
}

}  // namespace

extern "C" {

int stro_uq_stat(const double* values, int64_t n, int32_t max_batches, int32_t min_batches,
                 stro_stat_uq* out) {
    if (!out || (n > 0 && !values)) return fail(STRO_ERR_INVALID, "null argument");
    if (min_batches < 2 || max_batches < min_batches)
        return fail(STRO_ERR_INVALID, "batch counts: 2 <= min_batches <= max_batches");
    std::memset(out, 0, sizeof *out);
    if (n < int64_t(min_batches) * 4) {  // too short: mean only
        double s = 0.0;
        for (int64_t k = 0; k < n; ++k) s += values[k];
        out->mean = n > 0 ? s / double(n) : kNaN;
        out->half_width95 = kNaN;
        out->batches = 0;
        out->lag1 = kNaN;
        out->trustworthy = 0;
        return STRO_OK;
    }
    // search downward from max_batches (fewer, longer batches) for the largest
    // batch count whose means are effectively uncorrelated (Uncertainty.swift:89-99)
    bool chosen = false;
    for (int M = max_batches; M >= min_batches; M -= 2) {
        double mean, half, rho;
        batch_stats(values, n, M, &mean, &half, &rho);
        if (std::fabs(rho) <= 0.3) {
            out->batches = M;
            out->mean = mean;
            out->half_width95 = half;
            out->lag1 = rho;
            chosen = true;
            break;
        }
    }
    if (!chosen) {
        double mean, half, rho;
        batch_stats(values, n, min_batches, &mean, &half, &rho);
        out->batches = min_batches;
        out->mean = mean;
        out->half_width95 = half;
        out->lag1 = rho;
    }
    out->trustworthy = (out->batches >= 6 && std::fabs(out->lag1) <= 0.3) ? 1 : 0;
    return STRO_OK;
}

int stro_uq_num(const stro_ladder_rung* rungs_in, int32_t count, stro_num_uq* out) {
    if (!out || (count > 0 && !rungs_in)) return fail(STRO_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof *out);
    std::vector<stro_ladder_rung> r(rungs_in, rungs_in + count);
    // sorted by cells per feature (stable: equal resolutions keep their order)
    for (size_t i = 1; i < r.size(); ++i)
        for (size_t j = i; j > 0 && r[j].cells_per_feature < r[j - 1].cells_per_feature; --j)
            std::swap(r[j], r[j - 1]);
    out->observed_order = kNaN;
    if (count < 2) {
        out->u_num = kNaN;
        out->note = 0;  // single resolution
        return STRO_OK;
    }
    const stro_ladder_rung& fine = r[r.size() - 1];
    const stro_ladder_rung& mid = r[r.size() - 2];
    const double delta = std::fabs(fine.value - mid.value);
    const double fine_stat = std::isnan(fine.stat) ? 0.0 : fine.stat;
    out->u_num = smax(delta, fine_stat);
    if (count >= 3) {
        const stro_ladder_rung& c = r[r.size() - 3];
        const double d1 = mid.value - c.value;
        const double d2 = fine.value - mid.value;
        if (d1 * d2 > 0 && std::fabs(d2) < std::fabs(d1) && std::fabs(d2) > 0) {
            const double ratio = double(fine.cells_per_feature) / double(mid.cells_per_feature);
            if (ratio > 1.05) {
                out->observed_order = std::log(std::fabs(d1 / d2)) / std::log(ratio);
                out->has_order = 1;
            }
        }
    }
    out->note = delta <= fine_stat ? 1 : 2;
    return STRO_OK;
}

int stro_uq_mach(double baseline, double half_mach, double* u_ma) {
    if (!u_ma) return fail(STRO_ERR_INVALID, "null argument");
    // error ~ Ma^2: shift = e - e/4 = 3e/4, so e = 4/3 * shift (Uncertainty.swift:175-177)
    *u_ma = std::fabs(baseline - half_mach) * 4.0 / 3.0;
    return STRO_OK;
}

int stro_uq_classify(double re, double mach, int32_t cells_per_feature, const char* geometry,
                     stro_domain_verdict* out) {
    if (!out || !geometry) return fail(STRO_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof *out);
    int best = -1;
    double best_d = 0.0;
    for (int k = 0; k < kNumAnchors; ++k) {
        const Anchor& a = kAnchors[k];
        if (std::strcmp(a.geometry, geometry) != 0) continue;
        const double d_re = distance(re, a.re_lo, a.re_hi);
        const double d_ma = distance(mach, a.ma_lo, a.ma_hi);
        const double d_n = distance(double(cells_per_feature), double(a.n_lo), double(a.n_hi));
        const double d = smax(d_re, smax(d_ma, d_n));
        if (best < 0 || d < best_d) {
            best = k;
            best_d = d;
        }
    }
    out->anchor = best;
    if (best < 0) {
        out->verdict = STRO_DOMAIN_OUTSIDE;
        out->reasons = STRO_OUTSIDE_GEOMETRY;
        out->distance = kNaN;
        out->factor = kNaN;
        return STRO_OK;
    }
    out->distance = best_d;
    if (best_d == 0.0) {
        out->verdict = STRO_DOMAIN_INSIDE;
        out->factor = 1.0;
        return STRO_OK;
    }
    if (best_d <= 0.5) {
        out->verdict = STRO_DOMAIN_NEAR_EDGE;
        out->factor = 1.0 + 2.0 * best_d;
        return STRO_OK;
    }
    const Anchor& a = kAnchors[best];
    out->verdict = STRO_DOMAIN_OUTSIDE;
    out->factor = kNaN;
    if (distance(re, a.re_lo, a.re_hi) > 0) out->reasons |= STRO_OUTSIDE_RE;
    if (distance(mach, a.ma_lo, a.ma_hi) > 0) out->reasons |= STRO_OUTSIDE_MACH;
    if (distance(double(cells_per_feature), double(a.n_lo), double(a.n_hi)) > 0)
        out->reasons |= STRO_OUTSIDE_RESOLUTION;
    return STRO_OK;
}

int stro_uq_anchor(int32_t index, char* name, size_t name_len, double ranges[4],
                   int32_t cells[2], char* geometry, size_t geometry_len) {
    if (index < 0 || index >= kNumAnchors) return fail(STRO_ERR_INVALID, "no such anchor");
    const Anchor& a = kAnchors[index];
    if (name && name_len) {
        std::strncpy(name, a.name, name_len - 1);
        name[name_len - 1] = '\0';
    }
    if (ranges) {
        ranges[0] = a.re_lo;
        ranges[1] = a.re_hi;
        ranges[2] = a.ma_lo;
        ranges[3] = a.ma_hi;
    }
    if (cells) {
        cells[0] = a.n_lo;
        cells[1] = a.n_hi;
    }
    if (geometry && geometry_len) {
        std::strncpy(geometry, a.geometry, geometry_len - 1);
        geometry[geometry_len - 1] = '\0';
    }
    return STRO_OK;
}

int stro_uq_combined(double u_num, double u_stat, double u_ma, const stro_domain_verdict* v,
                     double* combined) {
    if (!v || !combined) return fail(STRO_ERR_INVALID, "null argument");
    // root sum of squares of the components that exist (Uncertainty.swift:272-280)
    double rss2 = 0.0;
    for (double p : {u_num, u_stat, u_ma})
        if (!std::isnan(p)) rss2 = rss2 + p * p;
    const double rss = std::sqrt(rss2);
    if (v->verdict == STRO_DOMAIN_INSIDE) *combined = 2.0 * rss;
    else if (v->verdict == STRO_DOMAIN_NEAR_EDGE) *combined = 2.0 * rss * v->factor;
    else *combined = kNaN;  // outside: no calibrated bar is published
    return STRO_OK;
}

}  // extern "C"
