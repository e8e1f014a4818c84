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

}  // namespace st
