// TEST INFRASTRUCTURE ONLY -- the oracle's dispersion: Cauchy's index (spectral.js:121-128 cauchyN), the
// wavelength's 15-bit code (spectral.js:136-137 lambdaCode / lambdaOf, :188-194 withLambda), and the camera's
// wavelength draw (lightspectra.js specDraw over CAMERA_TABLE: 1 nm cells of 380-780 nm, each drawn with its share
// of the three clipped Rec.709 colour-matching functions, each channel normalised to 1; the cell's colour is its
// weights over that share; the wavelength uniform in the cell from the same number).
//
// The colour-matching functions are the CIE 1931 observer's as fitted by Wyman, Sloan and Shirley (JCGT 2(2), 2013,
// the multi-lobe piecewise Gaussian), where the reference integrates the tabulated functions (its cie1931.js).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "st_oracle_core.h"

namespace sto {

const int SPEC_N = 400;                      // 1 nm cells from 380 nm
const double LD = 587.56, LF = 486.13, LC = 656.27;

// spectral.js cauchyN: n_d - B / lambda_d^2 + B / lambda^2 with B = (n_d - 1) / (V_d (1/lambda_F^2 - 1/lambda_C^2))
template <class T> inline T cauchy_n(T nd, T vd, T lam) {
    if (!(vd > T(0))) return nd;
    const T fc = T(1.0 / (LF * LF) - 1.0 / (LC * LC));
    const T B = (nd - T(1)) / (vd * fc);
    return nd + B * (T(1) / (lam * lam) - T(1) / T(LD * LD));
}
// the code a ray's tag keeps and the wavelength it reads back: 1 + round(clamp((l - 380) / 400) * 32766)
inline uint32_t lambda_code(double l) {
    double t = (l - 380.0) / 400.0;
    t = t < 0 ? 0 : (t > 1 ? 1 : t);
    return 1u + (uint32_t)std::nearbyint(t * 32766.0);
}
inline double lambda_of(uint32_t c) { return c ? 380.0 + (c - 1) * 400.0 / 32766.0 : 0.0; }
template <class T> inline T lambda_coded(T l) {
    const T c = T(1) + std::nearbyint(std::min(std::max((l - T(380)) / T(400), T(0)), T(1)) * T(32766));
    return T(380) + (c - T(1)) * (T(400) / T(32766));
}

struct SpecTable {
    float cdf[SPEC_N];
    float col[SPEC_N][3];
    SpecTable() {
        auto lobe = [](double l, double mu, double lo, double hi) {
            double t = (l - mu) / (l < mu ? lo : hi);
            return std::exp(-0.5 * t * t);
        };
        double w[SPEC_N][3] = {};
        double tot[3] = {0, 0, 0};
        for (int i = 0; i < SPEC_N; i++) {
            for (int k = 0; k < 8; k++) {                                        // 8 midpoints a cell
                double l = 380.0 + i + (k + 0.5) / 8.0;
                double X = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) -
                           0.065 * lobe(l, 501.1, 20.4, 26.2);
                double Y = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
                double Z = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
                double rgb[3] = {3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z,
                                 -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z,
                                 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z};
                for (int c = 0; c < 3; c++) w[i][c] += (rgb[c] > 0 ? rgb[c] : 0.0) / 8.0;
            }
            for (int c = 0; c < 3; c++) tot[c] += w[i][c];
        }
        double acc = 0;
        for (int i = 0; i < SPEC_N; i++) {
            double r = w[i][0] / tot[0], g = w[i][1] / tot[1], b = w[i][2] / tot[2];
            double q = (r + g + b) / 3.0;
            acc += q;
            cdf[i] = i == SPEC_N - 1 ? 1.0f : (float)acc;
            col[i][0] = (float)(q > 0 ? r / q : 0.0);
            col[i][1] = (float)(q > 0 ? g / q : 0.0);
            col[i][2] = (float)(q > 0 ? b / q : 0.0);
        }
    }
};
inline const SpecTable& spec_table() {
    static const SpecTable t;
    return t;
}

// A COATING (spectral.js:58-117, materials.js:150-163 coatMaterial). Its bins: 40 of 10 nm from 380 nm, per bin and
// channel the clipped Rec.709 colour-matching function's mean over the bin by the midpoint rule at 0.1 nm (spectral.js
// SPEC_WEIGHTS), each channel normalised to sum to 1.
struct CoatBins {
    double w[40][3];
    CoatBins() {
        auto lobe = [](double l, double mu, double lo, double hi) {
            double t = (l - mu) / (l < mu ? lo : hi);
            return std::exp(-0.5 * t * t);
        };
        double tot[3] = {0, 0, 0};
        for (int k = 0; k < 40; k++) {
            double a[3] = {0, 0, 0};
            for (int j = 0; j < 100; j++) {
                const double l = 380.0 + (k + (j + 0.5) / 100.0) * 10.0;
                const double X = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) -
                                 0.065 * lobe(l, 501.1, 20.4, 26.2);
                const double Y = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
                const double Z = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
                const double rgb[3] = {3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z,
                                       -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z,
                                       0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z};
                for (int c = 0; c < 3; c++) a[c] += (rgb[c] > 0 ? rgb[c] : 0.0) / 100.0;
            }
            for (int c = 0; c < 3; c++) { w[k][c] = a[c]; tot[c] += a[c]; }
        }
        for (int k = 0; k < 40; k++)
            for (int c = 0; c < 3; c++) w[k][c] /= tot[c];
    }
};
inline const CoatBins& coat_bins() {
    static const CoatBins b;
    return b;
}
// the logistic's scale s for a 10-90 % width (nm): width / (2 ln 9), the width at least 0.01 nm
inline double coat_scale(double width) { return std::max(width, 0.01) / (2.0 * std::log(9.0)); }
inline double softplus(double x) { return std::max(x, 0.0) + std::log1p(std::exp(-std::fabs(x))); }
// spectral.js edgeRGB: R(lambda) = lo + (hi - lo) / (1 + exp(-(lambda - edge) / s)) against each channel's bins, a bin's
// mean of the logistic exactly: s (softplus((b1 - edge) / s) - softplus((b0 - edge) / s)) / 10
inline void coat_edge_rgb(double lo, double hi, double edge, double width, double out[3]) {
    const CoatBins& B = coat_bins();
    const double s = coat_scale(width);
    double acc[3] = {0, 0, 0};
    for (int k = 0; k < 40; k++) {
        const double m = s * (softplus((390.0 + 10.0 * k - edge) / s) - softplus((380.0 + 10.0 * k - edge) / s)) / 10.0;
        for (int c = 0; c < 3; c++) acc[c] += B.w[k][c] * m;
    }
    for (int c = 0; c < 3; c++) out[c] = lo + (hi - lo) * acc[c];
}
// spectral.js edgeAt1: R at one wavelength
inline double coat_edge_at_lambda(double lo, double hi, double edge, double width, double lam) {
    return lo + (hi - lo) / (1.0 + std::exp(-(lam - edge) / coat_scale(width)));
}
// spectral.js edgeAt: the edge for light of invariant n0 sin(theta0) through a stack of effective index nEff
inline double coat_edge_at(double edge0, double nSin, double nEff) {
    const double q = nSin / std::max(nEff, 1e-6);
    return edge0 * std::sqrt(std::max(0.0, 1.0 - q * q));
}
// the draw: the first cell whose CDF passes u, the wavelength uniform in it from the same u
template <class T> inline T spec_draw(T u, V3<T>& w) {
    const SpecTable& t = spec_table();
    int lo = 0, hi = SPEC_N - 1;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (T(t.cdf[mid]) > u) hi = mid;
        else lo = mid + 1;
    }
    T c0 = lo ? T(t.cdf[lo - 1]) : T(0);
    T q = T(t.cdf[lo]) - c0;
    T f = q > T(0) ? std::min(std::max((u - c0) / q, T(0)), T(1)) : T(0.5);
    w = V3<T>(T(t.col[lo][0]), T(t.col[lo][1]), T(t.col[lo][2]));
    return T(380) + T(lo) + f;
}

}  // namespace sto
