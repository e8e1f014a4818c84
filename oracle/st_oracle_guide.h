// TEST INFRASTRUCTURE ONLY -- the oracle's restatement of the learned proposal (the product's st_guide.cuh and
// st_guide.cu): the hash-grid and spherical-harmonic input, the 48 -> 64 -> 64 -> 64 -> 40 network, the mixture of
// von Mises-Fisher lobes it decodes to, the training loss and its gradient with respect to every weight and feature.
// The reference has no counterpart (it removed its path guiding), so this pins the build against its own
// mathematics: evaluated in double it is the exact function, for finite-difference checks of the gradient; with BF16
// rounding at the points where the tensor cores take BF16 operands (the inputs, the weights, each hidden layer after
// its ReLU, the loss's gradient at the outputs and each hidden layer's gradient) it is what the GPU computes, up to
// the order of the FP32 sums.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace sto {
namespace guide {

const int LEVELS = 16, T = 1 << 12, IN = 48, H = 64, OUT = 40, LOBES = 8;
const int W1 = 0, W2 = W1 + H * IN, W3 = W2 + H * H, W4 = W3 + H * H, NW = W4 + OUT * H;
const int NHASH = LEVELS * T * 2, NPARAM = NW + NHASH;
const double KLO = -1.0, KHI = 6.0, WCAP = 1000.0;
const float RES[LEVELS] = {2, 2, 2, 3, 4, 5, 6, 7, 8, 10, 12, 15, 18, 22, 26, 32};

// round to the nearest BF16, ties to even (the finite values the network meets)
inline float bf16(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b += 0x7fffu + ((b >> 16) & 1u);
    b &= 0xffff0000u;
    float y;
    std::memcpy(&y, &b, 4);
    return y;
}
inline uint32_t hash3(uint32_t x, uint32_t y, uint32_t z) {
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (uint32_t)(T - 1);
}
// one level's 8 corner entries and trilinear weights at u in [0,1]^3 (f32, as the device computes them)
inline void corners(const float* u, int l, uint32_t* idx, float* w) {
    const float r = RES[l];
    float t[3];
    uint32_t c[3];
    for (int a = 0; a < 3; a++) {
        const float p = u[a] * r, f = std::floor(p);
        t[a] = p - f;
        c[a] = (uint32_t)(int32_t)f;
    }
    for (int k = 0; k < 8; k++) {
        const uint32_t ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
        idx[k] = (uint32_t)l * T + hash3(c[0] + ox, c[1] + oy, c[2] + oz);
        const float wx = ox ? t[0] : 1.f - t[0], wy = oy ? t[1] : 1.f - t[1], wz = oz ? t[2] : 1.f - t[2];
        w[k] = wx * wy * wz;
    }
}
inline void unit(const float* p, const float* lo, float inv_ext, float* u) {
    for (int a = 0; a < 3; a++) u[a] = std::fmin(std::fmax((p[a] - lo[a]) * inv_ext, 0.f), 1.f);
}
inline void sh16(double x, double y, double z, double* o) {
    const double xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814;
    o[1] = -0.48860251190291987 * y;
    o[2] = 0.48860251190291987 * z;
    o[3] = -0.48860251190291987 * x;
    o[4] = 1.0925484305920792 * x * y;
    o[5] = -1.0925484305920792 * y * z;
    o[6] = 0.94617469575755997 * zz - 0.31539156525251999;
    o[7] = -1.0925484305920792 * x * z;
    o[8] = 0.54627421529603959 * (xx - yy);
    o[9] = 0.59004358992664352 * y * (3 * xx - yy);
    o[10] = 2.8906114426405538 * x * y * z;
    o[11] = 0.45704579946446572 * y * (5 * zz - 1);
    o[12] = 0.3731763325901154 * z * (5 * zz - 3);
    o[13] = 0.45704579946446572 * x * (5 * zz - 1);
    o[14] = 1.4453057213202769 * z * (xx - yy);
    o[15] = 0.59004358992664352 * x * (xx - 3 * yy);
}

// one point's forward pass, keeping what the backward pass needs
struct Fwd {
    float u[3];
    uint32_t idx[LEVELS][8];
    float w[LEVELS][8];
    double x[IN], h1[H], h2[H], h3[H], y[OUT];
};
template <bool BF>
inline double q(double v) { return BF ? (double)bf16((float)v) : v; }

template <bool BF>
void forward(const float* P, const float* pos, const float* nrm, const float* lo, float inv_ext, Fwd& f) {
    unit(pos, lo, inv_ext, f.u);
    for (int l = 0; l < LEVELS; l++) {
        corners(f.u, l, f.idx[l], f.w[l]);
        double a = 0, b = 0;
        for (int k = 0; k < 8; k++) {
            a += (double)f.w[l][k] * P[NW + 2 * f.idx[l][k]];
            b += (double)f.w[l][k] * P[NW + 2 * f.idx[l][k] + 1];
        }
        f.x[2 * l] = q<BF>(a);
        f.x[2 * l + 1] = q<BF>(b);
    }
    double s[16];
    sh16(nrm[0], nrm[1], nrm[2], s);
    for (int k = 0; k < 16; k++) f.x[32 + k] = q<BF>(s[k]);
    auto layer = [&](const double* in, int nin, int off, int nout, double* out, bool relu) {
        for (int o = 0; o < nout; o++) {
            double acc = 0;
            for (int i = 0; i < nin; i++) acc += in[i] * q<BF>(P[off + o * nin + i]);
            out[o] = relu ? q<BF>(std::fmax(acc, 0.0)) : acc;
        }
    };
    layer(f.x, IN, W1, H, f.h1, true);
    layer(f.h1, H, W2, H, f.h2, true);
    layer(f.h2, H, W3, H, f.h3, true);
    layer(f.h3, H, W4, OUT, f.y, false);
}

// the mixture the outputs decode to: mean directions, kappa = e^clamp(log kappa), weights by softmax (exact)
inline void decode(const double* y, double (*mix)[5]) {
    double mx = -1e300, s = 0, e[LOBES];
    for (int k = 0; k < LOBES; k++) mx = std::fmax(mx, y[5 * k + 4]);
    for (int k = 0; k < LOBES; k++) { e[k] = std::exp(y[5 * k + 4] - mx); s += e[k]; }
    for (int k = 0; k < LOBES; k++) {
        double m[3] = {y[5 * k], y[5 * k + 1], y[5 * k + 2]};
        double l = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        if (l <= 1e-12) { m[0] = 0; m[1] = 0; m[2] = 1; l = 1; }
        for (int a = 0; a < 3; a++) mix[k][a] = m[a] / l;
        mix[k][3] = std::exp(std::fmin(std::fmax(y[5 * k + 3], KLO), KHI));
        mix[k][4] = e[k] / s;
    }
}
// the vMF density at cos c: kappa / (2 pi (1 - e^-2 kappa)) e^(kappa (c - 1))
inline double vmf_pdf(double kappa, double c) {
    return kappa / (2 * M_PI * (-std::expm1(-2 * kappa))) * std::exp(kappa * (c - 1));
}
inline double mix_pdf(const double (*mix)[5], const double* d) {
    double p = 0;
    for (int k = 0; k < LOBES; k++)
        p += mix[k][4] * vmf_pdf(mix[k][3], mix[k][0] * d[0] + mix[k][1] * d[1] + mix[k][2] * d[2]);
    return p;
}
// a direction from the mixture with the numbers (u0, u1, u2): the lobe by weight, then the vMF draw
inline void mix_sample(const double (*mix)[5], double u0, double u1, double u2, double* d) {
    int k = LOBES - 1;
    double acc = 0;
    for (int j = 0; j + 1 < LOBES; j++) { acc += mix[j][4]; if (u0 < acc) { k = j; break; } }
    const double kap = mix[k][3];
    const double c = std::fmin(std::fmax(1 + std::log(u1 + (1 - u1) * std::exp(-2 * kap)) / kap, -1.0), 1.0);
    const double s = std::sqrt(std::fmax(0.0, 1 - c * c));
    const double* mu = mix[k];
    double t1[3];
    if (std::fabs(mu[2]) < 0.999) { t1[0] = mu[1]; t1[1] = -mu[0]; t1[2] = 0; }      // mu x z
    else { t1[0] = -mu[2]; t1[1] = 0; t1[2] = mu[0]; }                                  // mu x y
    const double l = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (int a = 0; a < 3; a++) t1[a] /= l;
    const double t2[3] = {mu[1] * t1[2] - mu[2] * t1[1], mu[2] * t1[0] - mu[0] * t1[2], mu[0] * t1[1] - mu[1] * t1[0]};
    const double ph = 2 * M_PI * u2;
    for (int a = 0; a < 3; a++) d[a] = mu[a] * c + t1[a] * (s * std::cos(ph)) + t2[a] * (s * std::sin(ph));
    const double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int a = 0; a < 3; a++) d[a] /= n;
}

// -w log q(d) and its gradient at the 40 outputs
inline double loss_grad(const double* y, const double* d, double w, double* dy) {
    double mx = -1e300, s = 0, pi[LOBES];
    for (int k = 0; k < LOBES; k++) mx = std::fmax(mx, y[5 * k + 4]);
    for (int k = 0; k < LOBES; k++) { pi[k] = std::exp(y[5 * k + 4] - mx); s += pi[k]; }
    double lv[LOBES], kap[LOBES], cs[LOBES], len[LOBES], mu[LOBES][3], lmax = -1e300;
    for (int k = 0; k < LOBES; k++) {
        pi[k] /= s;
        const double m[3] = {y[5 * k], y[5 * k + 1], y[5 * k + 2]};
        len[k] = std::fmax(std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]), 1e-12);
        for (int a = 0; a < 3; a++) mu[k][a] = m[a] / len[k];
        kap[k] = std::exp(std::fmin(std::fmax(y[5 * k + 3], KLO), KHI));
        cs[k] = mu[k][0] * d[0] + mu[k][1] * d[1] + mu[k][2] * d[2];
        lv[k] = std::log(kap[k]) - std::log(2 * M_PI) - std::log(-std::expm1(-2 * kap[k])) + kap[k] * (cs[k] - 1) +
                std::log(pi[k]);
        lmax = std::fmax(lmax, lv[k]);
    }
    double acc = 0;
    for (int k = 0; k < LOBES; k++) acc += std::exp(lv[k] - lmax);
    const double lq = lmax + std::log(acc);
    for (int k = 0; k < LOBES; k++) {
        const double r = std::exp(lv[k] - lq);
        const double e2 = std::exp(-2 * kap[k]);
        const double dk = 1 / kap[k] - 2 * e2 / (1 - e2) + (cs[k] - 1);
        const double kr = y[5 * k + 3];
        const double inr = (kr > KLO && kr < KHI) ? 1 : 0;
        const double gm = -w * r * kap[k] / len[k];
        for (int a = 0; a < 3; a++) dy[5 * k + a] = gm * (d[a] - mu[k][a] * cs[k]);
        dy[5 * k + 3] = -w * r * dk * kap[k] * inr;
        dy[5 * k + 4] = -w * (r - pi[k]);
    }
    return -w * lq;
}

// the batch's loss and its gradient with respect to every parameter (G: NPARAM, added to), each sample's weight
// over the batch's mean, capped
template <bool BF>
double batch_grad(const float* P, int n, const float* pos, const float* nrm, const float* dir, const float* wt,
                  const float* lo, float inv_ext, double* G) {
    double wsum = 0;
    for (int i = 0; i < n; i++) wsum += wt[i];
    const float mean = (float)wsum / (float)n;                          // as the device: an FP32 sum over an FP32 count
    const double inv_mean = mean > 0 ? 1.0 / (double)mean : 0.0;
    double loss = 0;
    Fwd f;
    for (int i = 0; i < n; i++) {
        forward<BF>(P, pos + 3 * i, nrm + 3 * i, lo, inv_ext, f);
        const double w = std::fmin((double)wt[i] * inv_mean, WCAP);
        double dy[OUT];
        const double d[3] = {dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
        loss += loss_grad(f.y, d, w, dy);
        for (int o = 0; o < OUT; o++) dy[o] = q<BF>(dy[o]);
        // backward through W4, W3, W2 (masked by each ReLU), then W1 to the inputs
        double d3[H], d2[H], d1[H], dx[IN];
        auto back = [&](const double* dz, int nz, int off, int nin, const double* act, double* out, bool mask) {
            for (int i2 = 0; i2 < nin; i2++) {
                double acc = 0;
                for (int o = 0; o < nz; o++) acc += dz[o] * q<BF>(P[off + o * nin + i2]);
                out[i2] = mask ? (act[i2] > 0 ? q<BF>(acc) : 0.0) : acc;
            }
            for (int o = 0; o < nz; o++)
                for (int i2 = 0; i2 < nin; i2++) G[off + o * nin + i2] += dz[o] * act[i2];
        };
        back(dy, OUT, W4, H, f.h3, d3, true);
        back(d3, H, W3, H, f.h2, d2, true);
        back(d2, H, W2, H, f.h1, d1, true);
        back(d1, H, W1, IN, f.x, dx, false);
        for (int l = 0; l < LEVELS; l++)
            for (int k = 0; k < 8; k++) {
                G[NW + 2 * f.idx[l][k]] += (double)f.w[l][k] * dx[2 * l];
                G[NW + 2 * f.idx[l][k] + 1] += (double)f.w[l][k] * dx[2 * l + 1];
            }
    }
    return loss;
}

}  // namespace guide
}  // namespace sto
