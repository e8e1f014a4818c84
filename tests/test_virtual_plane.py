"""The lux plane from the far field (optics.py virtual_plane, the reference's optics/illum.js:206-248 virtualPlane): the
luminaire taken as a point, E = I(gamma, C) cos^3(gamma) / h^2, I bilinear on the type C grid. Checked on the far field
of a Lambertian point source, I = I0 cos(gamma) over the lower hemisphere, whose plane reads I0 cos^4(gamma) / h^2."""
import math

import numpy as np

from shadytracer_gb300.optics import virtual_plane, intensity


def lambertian_far(nC, nG, flux=1000.0):
    """The far field of a Lambertian emitter of `flux` lumens as the tally holds it: flux a bin (gamma 0 the axis)."""
    dG = 180.0 / (nG - 1)
    j = np.arange(nG)
    lo = np.radians(np.maximum(0.0, (j - 0.5) * dG))
    hi = np.radians(np.minimum(180.0, (j + 0.5) * dG))
    # the flux between two cones of a Lambertian emitter: flux (sin^2 hi - sin^2 lo), within 90 degrees
    s2 = lambda a: np.sin(np.minimum(a, math.pi / 2)) ** 2
    row = flux * (s2(hi) - s2(lo))
    return np.repeat(row[:, None] / nC, nC, axis=1)


def test_the_far_field_of_a_lambertian_source_is_its_intensity():
    nC, nG = 360, 181
    far = lambertian_far(nC, nG)
    I = intensity(far, nC, nG)
    I0 = 1000.0 / math.pi
    g = np.radians(np.arange(nG) * 180.0 / (nG - 1))
    inner = (g > 0.05) & (g < math.radians(85))
    assert np.allclose(I[inner, 0], I0 * np.cos(g[inner]), rtol=2e-4)
    assert abs((far.sum() - 1000.0)) < 1e-9


def test_the_virtual_plane_of_a_lambertian_source():
    nC, nG, h, half, cells = 360, 181, 1.0, 1.0, 64
    I = intensity(lambertian_far(nC, nG), nC, nG)
    E = virtual_plane(I, nC, nG, h=h, half=half, cells=cells)
    c = -half + (np.arange(cells) + 0.5) * (2 * half / cells)
    a, b = np.meshgrid(c, c)
    cg = h / np.sqrt(h * h + a * a + b * b)
    exact = 1000.0 / math.pi * cg ** 4 / (h * h)
    assert np.allclose(E, exact, rtol=2e-3)
    cell = 2 * half / cells
    assert abs((E * cell * cell).sum() / (exact * cell * cell).sum() - 1) < 1e-3
