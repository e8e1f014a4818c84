// st_sky.h -- the physical sun and sky's host half (core/environment.js SKY_BAND_TABLE, SUNSKY_FN): the sixteen bands
// of the spectrum, 380 to 730 nm, that the device's sun and sky adds up as colour, built once in double.
//
// A BAND k covers [380 + 21.875 k, 380 + 21.875 (k + 1)) nm, sampled at every nanometre from its start. Its weights are
// sunlight above the air (Planck's law at 5778 K, the sun's effective temperature) times the CIE 1931 colour-matching
// functions (the Wyman-Sloan-Shirley fit of st_spectral.h; the reference integrates the tabulated functions, which the
// fit follows to about 1 % of their peaks), taken to linear Rec.709 (the XYZ -> sRGB matrix); the sixteen colours are
// scaled together so they sum to luminance 1. Its middle is the wavelength weighted by the light (x + y + z). There:
//   the Rayleigh optical depth of the whole atmosphere straight up, 0.008569 l^-4 (1 + 0.0113 l^-2 + 0.00013 l^-4),
//     l in micrometres (Hansen & Travis 1974, Space Sci. Rev. 16, eq. 2.29);
//   the aerosol's depth per unit of its depth at 550 nm, Angstrom's law (l / 550)^-1.3;
//   the ozone's depth for a 300 Dobson-unit column (2.6867e16 molecules a cm^2 a unit), absorbed only: the Chappuis
//     band's cross-section per band at 223 K (Serdyuchenko, Gorshelev, Weber et al. 2014, AMT 7, the IUP Bremen data as
//     the reference averages it over each band).
#pragma once
#include <cmath>
#include <vector>

#include "st_spectral.h"

namespace st {

constexpr int SKY_BANDS = 16;
constexpr double SKY_LO_NM = 380.0, SKY_HI_NM = 730.0;

// per band (cm^2 a molecule): the Chappuis band's cross-section, 223 K
constexpr double SKY_OZONE_SIGMA[SKY_BANDS] = {6.2648e-24, 3.1169e-23, 1.0195e-22, 2.4886e-22, 5.4883e-22, 1.1517e-21,
                                               2.0211e-21, 3.0497e-21, 4.2480e-21, 4.5252e-21, 4.7153e-21, 3.4726e-21,
                                               2.3885e-21, 1.5936e-21, 9.8370e-22, 6.3061e-22};
constexpr double SKY_OZONE_COLUMN = 300.0 * 2.6867e16;

// the table as the device reads it: per band (Rayleigh depth, aerosol factor, ozone depth, middle nm), then per band
// (r, g, b, 0) -- 2 x 16 float4s' worth of doubles, in that order
inline std::vector<double> sky_band_table() {
    const double step = (SKY_HI_NM - SKY_LO_NM) / SKY_BANDS;
    std::vector<double> out(8 * SKY_BANDS, 0.0);
    double tot[3] = {0, 0, 0};
    std::vector<double> rgb(3 * SKY_BANDS);
    for (int k = 0; k < SKY_BANDS; k++) {
        double X = 0, Y = 0, Z = 0, wl = 0, ws = 0;
        for (double l = SKY_LO_NM + k * step; l < SKY_LO_NM + (k + 1) * step; l += 1.0) {
            const double li = std::round(l);                          // the colour-matching functions at whole nm
            const double m = l * 1e-9;
            const double w = 1.0 / (m * m * m * m * m * (std::exp(1.438776877e-2 / (m * 5778.0)) - 1.0));
            double x, y, z;
            cie_xyz_fit(li, x, y, z);
            X += w * x; Y += w * y; Z += w * z;
            wl += w * (x + y + z) * l;
            ws += w * (x + y + z);
        }
        const double nm = wl / ws, um = nm / 1000.0;
        out[4 * k + 0] = 0.008569 * std::pow(um, -4.0) * (1 + 0.0113 * std::pow(um, -2.0) + 0.00013 * std::pow(um, -4.0));
        out[4 * k + 1] = std::pow(nm / 550.0, -1.3);
        out[4 * k + 2] = SKY_OZONE_SIGMA[k] * SKY_OZONE_COLUMN;
        out[4 * k + 3] = nm;
        rgb[3 * k + 0] = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z;
        rgb[3 * k + 1] = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z;
        rgb[3 * k + 2] = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z;
        for (int c = 0; c < 3; c++) tot[c] += rgb[3 * k + c];
    }
    const double Yt = 0.2126 * tot[0] + 0.7152 * tot[1] + 0.0722 * tot[2];
    for (int k = 0; k < SKY_BANDS; k++)
        for (int c = 0; c < 3; c++) out[4 * SKY_BANDS + 4 * k + c] = rgb[3 * k + c] / Yt;
    return out;
}

}  // namespace st
