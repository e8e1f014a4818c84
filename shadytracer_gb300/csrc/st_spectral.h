// st_spectral.h -- dispersion's host half: the camera's wavelength table (lightspectra.js CAMERA_TABLE, specDraw)
// and Cauchy's index (spectral.js cauchyN), for st_capi.cu (the table is built once a context, in double, and
// uploaded as SPEC_CELLS float4s: the draw's CDF and each cell's colour per channel).
//
// THE TABLE. 400 cells of 1 nm from 380 nm. A cell's weight in each Rec.709 channel is the integral over the cell of
// that channel's colour-matching function, negative parts clipped to 0, each channel normalised to sum to 1 over the
// cells; a cell is drawn with probability q_i, the mean of its three weights, and its colour is the weights over q_i
// -- so each channel's mean over the draw is exactly 1 and no channel exceeds 3. The colour-matching functions are
// the CIE 1931 2-degree observer's as fitted by Wyman, Sloan and Shirley ("Simple Analytic Approximations to the CIE
// XYZ Color Matching Functions", JCGT 2(2), 2013, the multi-lobe piecewise-Gaussian fit), taken to linear Rec.709 by
// the standard XYZ -> sRGB (D65) matrix; the reference integrates the tabulated CIE functions instead (its
// cie1931.js), which the fit follows to within about 1 % of the peaks.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace st {

constexpr int SPEC_CELLS = 400;              // 1 nm cells, 380-780 nm (lightspectra.js)
constexpr double SPEC_LO_NM = 380.0;
constexpr double LAMBDA_D_NM = 587.56, LAMBDA_F_NM = 486.13, LAMBDA_C_NM = 656.27;   // spectral.js Fraunhofer lines
constexpr int LAMBDA_STEPS = 32766;          // the wavelength's 15-bit code (spectral.js lambdaCode)

// one lobe of the fit: a Gaussian of a different width either side of its peak
inline double wss_lobe(double l, double mu, double s1, double s2) {
    const double t = (l - mu) / (l < mu ? s1 : s2);
    return std::exp(-0.5 * t * t);
}
inline void cie_xyz_fit(double l, double& x, double& y, double& z) {
    x = 1.056 * wss_lobe(l, 599.8, 37.9, 31.0) + 0.362 * wss_lobe(l, 442.0, 16.0, 26.7) -
        0.065 * wss_lobe(l, 501.1, 20.4, 26.2);
    y = 0.821 * wss_lobe(l, 568.8, 46.9, 40.5) + 0.286 * wss_lobe(l, 530.9, 16.3, 31.1);
    z = 1.217 * wss_lobe(l, 437.0, 11.8, 36.0) + 0.681 * wss_lobe(l, 459.0, 26.0, 13.8);
}
// each cell: (CDF up to and with the cell, colour r, g, b)
inline std::vector<double> spectral_table() {
    constexpr int SUB = 8;                                     // midpoint samples a cell
    std::vector<double> w(3 * SPEC_CELLS, 0.0);
    double sum[3] = {0, 0, 0};
    for (int i = 0; i < SPEC_CELLS; i++) {
        for (int k = 0; k < SUB; k++) {
            const double l = SPEC_LO_NM + i + (k + 0.5) / SUB;
            double X, Y, Z;
            cie_xyz_fit(l, X, Y, Z);
            const double r = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z;
            const double g = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z;
            const double b = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z;
            w[3 * i] += std::fmax(r, 0.0) / SUB;
            w[3 * i + 1] += std::fmax(g, 0.0) / SUB;
            w[3 * i + 2] += std::fmax(b, 0.0) / SUB;
        }
        for (int c = 0; c < 3; c++) sum[c] += w[3 * i + c];
    }
    std::vector<double> out(4 * SPEC_CELLS);
    double cdf = 0;
    for (int i = 0; i < SPEC_CELLS; i++) {
        const double r = w[3 * i] / sum[0], g = w[3 * i + 1] / sum[1], b = w[3 * i + 2] / sum[2];
        const double q = (r + g + b) / 3.0;
        cdf += q;
        out[4 * i] = i + 1 == SPEC_CELLS ? 1.0 : cdf;
        out[4 * i + 1] = q > 0 ? r / q : 0.0;
        out[4 * i + 2] = q > 0 ? g / q : 0.0;
        out[4 * i + 3] = q > 0 ? b / q : 0.0;
    }
    return out;
}

// A COATING'S BINS (spectral.js SPEC_WEIGHTS, what coat_edge_rgb in st_device.cuh averages a coating's R(lambda)
// against): COAT_BINS bins of 10 nm from 380 nm, per bin and channel the mean of the clipped Rec.709 colour-matching
// function over the bin (the midpoint rule at 0.1 nm), each channel normalised to sum to 1 over the bins -- so a
// constant R is that R in every channel exactly. Returned as COAT_BINS rows of (r, g, b).
constexpr int COAT_BINS = 40;
constexpr double COAT_STEP_NM = 10.0;
inline std::vector<double> coat_bin_table() {
    constexpr int SUB = 100;
    std::vector<double> w(3 * COAT_BINS, 0.0);
    double sum[3] = {0, 0, 0};
    for (int k = 0; k < COAT_BINS; k++) {
        for (int j = 0; j < SUB; j++) {
            const double l = SPEC_LO_NM + (k + (j + 0.5) / SUB) * COAT_STEP_NM;
            double X, Y, Z;
            cie_xyz_fit(l, X, Y, Z);
            const double c[3] = {3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z,
                                 -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z,
                                 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z};
            for (int i = 0; i < 3; i++) w[3 * k + i] += std::fmax(c[i], 0.0) / SUB;
        }
        for (int i = 0; i < 3; i++) sum[i] += w[3 * k + i];
    }
    for (int k = 0; k < COAT_BINS; k++)
        for (int i = 0; i < 3; i++) w[3 * k + i] /= sum[i];
    return w;
}

// THE TRACE BY WAVELENGTH's tables (optics/spectral.js SP_CDF_TABLE, SP_BASIS_TABLE, sourceSpectrum), on SPO_N nodes
// 1 nm apart from SPO_LO nm: the draw's CDF over p(l) = x-bar + y-bar + z-bar (each 1 nm cell carrying the mean of its
// two ends, so p is constant in a cell), the colour-matching functions, the basis an RGB colour becomes a spectrum by
// (the Rec.709 colour-matching functions clipped at 0 over their sum, 1/3 each where all are 0) -- and a light's
// spectrum at the nodes normalised to luminance 1 by the exact integral of two functions linear between the nodes.
constexpr int SPO_N = 471;
constexpr double SPO_LO = 360.0;
inline void spo_cmf(double l, double& x, double& y, double& z) { cie_xyz_fit(l, x, y, z); }
inline void xyz_to_rgb709(const double* c, double* rgb) {
    rgb[0] = 3.2404542 * c[0] - 1.5371385 * c[1] - 0.4985314 * c[2];
    rgb[1] = -0.9692660 * c[0] + 1.8760108 * c[1] + 0.0415560 * c[2];
    rgb[2] = 0.0556434 * c[0] - 0.2040259 * c[1] + 1.0572252 * c[2];
}
// cdf (SPO_N), cmf x y z (3 SPO_N), basis r g b (3 SPO_N)
inline std::vector<double> spo_tables() {
    std::vector<double> t(7 * SPO_N, 0.0);
    double* cdf = t.data();
    double* cmf = cdf + SPO_N;
    double* bas = cmf + 3 * SPO_N;
    std::vector<double> p(SPO_N);
    for (int i = 0; i < SPO_N; i++) {
        double c[3];
        spo_cmf(SPO_LO + i, c[0], c[1], c[2]);
        for (int k = 0; k < 3; k++) cmf[k * SPO_N + i] = c[k];
        p[i] = c[0] + c[1] + c[2];
        double rgb[3];
        xyz_to_rgb709(c, rgb);
        double sum = 0;
        for (int k = 0; k < 3; k++) { rgb[k] = std::fmax(rgb[k], 0.0); sum += rgb[k]; }
        for (int k = 0; k < 3; k++) bas[k * SPO_N + i] = sum > 0 ? rgb[k] / sum : 1.0 / 3.0;
    }
    cdf[0] = 0;
    for (int i = 1; i < SPO_N; i++) cdf[i] = cdf[i - 1] + 0.5 * (p[i - 1] + p[i]);
    for (int i = 1; i < SPO_N; i++) cdf[i] /= cdf[SPO_N - 1];
    cdf[SPO_N - 1] = 1.0;
    return t;
}
// the integral of two functions linear between the nodes, cell by cell exactly
inline double spo_integral(const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i + 1 < SPO_N; i++)
        s += (a[i] * b[i] + a[i + 1] * b[i + 1]) / 3.0 + (a[i] * b[i + 1] + a[i + 1] * b[i]) / 6.0;
    return s;
}
// A LIGHT'S SPECTRUM at the nodes, luminance 1: a table's row when given, else a blackbody of cct kelvin, else a
// stand-in of exactly the colour's XYZ made of the three basis spectra (white where the colour is 0 0 0)
inline std::vector<double> spo_source(const std::vector<double>& tab, const float* row, double cct, const float* colour) {
    std::vector<double> s(SPO_N, 0.0);
    const double* cmf = tab.data() + SPO_N;
    const double* bas = cmf + 3 * SPO_N;
    auto stand_in = [&](const double* rgb) {
        const double xyz[3] = {0.4124564 * rgb[0] + 0.3575761 * rgb[1] + 0.1804375 * rgb[2],
                               0.2126729 * rgb[0] + 0.7151522 * rgb[1] + 0.0721750 * rgb[2],
                               0.0193339 * rgb[0] + 0.1191920 * rgb[1] + 0.9503041 * rgb[2]};
        double M[3][3];                                     // XYZ = M w: column c the basis c's XYZ
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) M[r][c] = spo_integral(bas + c * SPO_N, cmf + r * SPO_N);
        const double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                           M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                           M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
        double inv[3][3];
        inv[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) / det;
        inv[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
        inv[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
        inv[1][0] = (M[1][2] * M[2][0] - M[1][0] * M[2][2]) / det;
        inv[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
        inv[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
        inv[2][0] = (M[1][0] * M[2][1] - M[1][1] * M[2][0]) / det;
        inv[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
        inv[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
        double w[3];
        for (int c = 0; c < 3; c++) w[c] = inv[c][0] * xyz[0] + inv[c][1] * xyz[1] + inv[c][2] * xyz[2];
        for (int i = 0; i < SPO_N; i++) s[i] = w[0] * bas[i] + w[1] * bas[SPO_N + i] + w[2] * bas[2 * SPO_N + i];
    };
    if (row) {
        for (int i = 0; i < SPO_N; i++) s[i] = std::fmax((double)row[i], 0.0);
    } else if (cct > 0) {
        for (int i = 0; i < SPO_N; i++) {
            const double m = (SPO_LO + i) * 1e-9;
            s[i] = 1e-30 / (m * m * m * m * m * std::expm1(1.4387769e-2 / (m * cct)));
        }
    } else {
        const bool zero = !(colour[0] != 0.f || colour[1] != 0.f || colour[2] != 0.f);
        const double rgb[3] = {zero ? 1.0 : colour[0], zero ? 1.0 : colour[1], zero ? 1.0 : colour[2]};
        stand_in(rgb);
    }
    double Y = spo_integral(s.data(), cmf + SPO_N);
    if (!(Y > 0)) {
        const double white[3] = {1, 1, 1};
        stand_in(white);
        Y = spo_integral(s.data(), cmf + SPO_N);
    }
    for (double& v : s) v /= Y;
    return s;
}

}  // namespace st
