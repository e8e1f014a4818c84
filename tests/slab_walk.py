"""TEST INFRASTRUCTURE: a slab walk in numpy -- the transmission of a beam at normal incidence through a slab of
optical depth tau whose faces do nothing (index-matched), scattering with Henyey-Greenstein's phase function of
asymmetry g and absorbing nothing: free flights of -ln(1 - u) optical lengths, each collision turning the ray, until
it leaves by either face (core/haze.js slabWalkJS, the walk core/test/volume.test.mjs holds to radiative transfer).
Returns the shares transmitted, reflected and never collided, and the mean number of collisions a ray takes."""
import numpy as np


def hg_cos(g, u):
    if abs(g) < 1e-3:
        return 1.0 - 2.0 * u
    s = (1.0 - g * g) / (1.0 - g + 2.0 * g * u)
    return np.clip((1.0 + g * g - s * s) / (2.0 * g), -1.0, 1.0)


def slab_walk(tau, g, rays=200_000, seed=11):
    r = np.random.default_rng(seed)
    z = np.zeros(rays)
    mu = np.ones(rays)                     # the direction's cosine to the slab's normal, into the slab
    alive = np.ones(rays, bool)
    through = np.zeros(rays, bool)
    collided = np.zeros(rays, bool)
    hits = np.zeros(rays)
    while alive.any():
        i = np.nonzero(alive)[0]
        z[i] += mu[i] * -np.log1p(-r.random(len(i)))
        out_t = z[i] >= tau
        out_r = z[i] <= 0.0
        through[i[out_t]] = True
        alive[i[out_t | out_r]] = False
        j = i[~(out_t | out_r)]
        if len(j) == 0:
            break
        collided[j] = True
        hits[j] += 1
        c = hg_cos(g, r.random(len(j)))
        phi = 2.0 * np.pi * r.random(len(j))
        s0 = np.sqrt(np.maximum(0.0, 1.0 - mu[j] ** 2))
        mu[j] = np.clip(mu[j] * c + s0 * np.sqrt(np.maximum(0.0, 1.0 - c * c)) * np.cos(phi), -1.0, 1.0)
    return {"T": through.mean(), "R": 1.0 - through.mean(), "ballistic": (~collided).mean(), "steps": hits.mean()}
