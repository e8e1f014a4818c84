"""TEST INFRASTRUCTURE: the closed forms the trace by wavelength is held to (optics/spectral.js; the reference's
optics-spectral rows, lib/pathtracer/tests.js:1469-1531), at the 1 nm nodes from 360 nm the trace reads its tables at:
the CIE 1931 colour-matching functions (Wyman, Sloan and Shirley's multi-lobe fit), a blackbody's spectrum, a stand-in
spectrum of exactly a colour's XYZ, and what a spectrum lets through a transmission T(l) -- its share of the luminous
flux and the colour that comes out."""
import math

import numpy as np

LO, N = 360.0, 471
L = LO + np.arange(N)


def cmf(l):
    g = lambda x, mu, s1, s2: np.exp(-0.5 * ((x - mu) / np.where(x < mu, s1, s2)) ** 2)
    x = 1.056 * g(l, 599.8, 37.9, 31.0) + 0.362 * g(l, 442.0, 16.0, 26.7) - 0.065 * g(l, 501.1, 20.4, 26.2)
    y = 0.821 * g(l, 568.8, 46.9, 40.5) + 0.286 * g(l, 530.9, 16.3, 31.1)
    z = 1.217 * g(l, 437.0, 11.8, 36.0) + 0.681 * g(l, 459.0, 26.0, 13.8)
    return np.stack([x, y, z])


CMF = cmf(L)
RGB_TO_XYZ = np.array([[0.4124564, 0.3575761, 0.1804375], [0.2126729, 0.7151522, 0.0721750],
                       [0.0193339, 0.1191920, 0.9503041]])
XYZ_TO_RGB = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
                       [0.0556434, -0.2040259, 1.0572252]])


def basis():
    rgb = np.maximum(XYZ_TO_RGB @ CMF, 0.0)
    s = rgb.sum(0)
    return np.where(s > 0, rgb / np.where(s > 0, s, 1), 1.0 / 3.0)


def integral(a, b):
    """Two functions linear between the nodes, integrated exactly."""
    return float(np.sum((a[:-1] * b[:-1] + a[1:] * b[1:]) / 3.0 + (a[:-1] * b[1:] + a[1:] * b[:-1]) / 6.0))


def planck(T):
    m = L * 1e-9
    return 1e-30 / (m ** 5 * np.expm1(1.4387769e-2 / (m * T)))


def stand_in(rgb):
    B = basis()
    M = np.array([[integral(B[c], CMF[r]) for c in range(3)] for r in range(3)])
    w = np.linalg.solve(M, RGB_TO_XYZ @ np.asarray(rgb, float))
    return w @ B


def normalised(s):
    return s / integral(s, CMF[1])


def xy(X):
    t = X[0] + X[1] + X[2]
    return np.array([X[0] / t, X[1] / t])


def through(s, T):
    """What spectrum s lets through a transmission T (an array at the nodes): (share of its luminous flux, xy out)."""
    s = normalised(s)
    X = np.array([np.sum(s * CMF[k] * T) for k in range(3)])
    return X[1] / np.sum(s * CMF[1]), xy(X)


def upvp(c):
    x, y = c
    d = -2 * x + 12 * y + 3
    return np.array([4 * x / d, 9 * y / d])


def duv(a, b):
    return float(np.linalg.norm(upvp(a) - upvp(b)))
