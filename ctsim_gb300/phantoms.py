"""Seeded synthetic phantoms for the benchmark configurations.

The reference's benchmarks run on its built-in phantoms; the fan-beam and
batched configurations use random-ellipse phantoms drawn here with
numpy.random.default_rng(seed): centres uniform in the unit disk, semi-axes
U[0.05, 0.5], rotation U[0, 180) degrees, attenuation U[-0.5, 1.0].  They can
be written as CTSim phantom files (`type cx cy u v rot atten` per line,
libctsim/phantom.cpp:184-213) so the reference reads the identical phantom.
"""
import numpy as np


def random_ellipses(seed, n=12):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        r = np.sqrt(rng.uniform(0.0, 1.0))
        t = rng.uniform(0.0, 2 * np.pi)
        u, v = rng.uniform(0.05, 0.5, size=2)
        rot = rng.uniform(0.0, 180.0)
        att = rng.uniform(-0.5, 1.0)
        out.append(("ellipse", float(r * np.cos(t)), float(r * np.sin(t)), float(u), float(v),
                    float(rot), float(att)))
    return out


def write_phm(path, elements):
    with open(path, "w") as f:
        for e in elements:
            f.write("%s %.17g %.17g %.17g %.17g %.17g %.17g\n" % e)


def make_phantom(elements):
    """A ctsim_gb300.Phantom holding `elements` (added in order)."""
    from . import Phantom
    p = Phantom()
    for e in elements:
        p.add_element(*e)
    return p


def random_ellipsoids(seed, n=16, z_half=1.0):
    """Seeded 3-D ellipsoid phantom: rows (cx, cy, cz, a, b, c, rot_deg, atten),
    the in-plane draws as random_ellipses (centres uniform in the unit disk,
    semi-axes U[0.05, 0.5], rotation U[0, 180) degrees, attenuation
    U[-0.5, 1.0]), z centres uniform in [-z_half, z_half] and z semi-axes
    U[0.05, 0.5] * 2 z_half."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n):
        r = np.sqrt(rng.uniform(0.0, 1.0))
        t = rng.uniform(0.0, 2 * np.pi)
        a, b = rng.uniform(0.05, 0.5, size=2)
        rot = rng.uniform(0.0, 180.0)
        att = rng.uniform(-0.5, 1.0)
        cz = rng.uniform(-z_half, z_half)
        c = rng.uniform(0.05, 0.5) * 2 * z_half
        rows.append((r * np.cos(t), r * np.sin(t), cz, a, b, c, rot, att))
    return np.array(rows, np.float64)


def ellipsoid_footprint(ellipsoids):
    """2-D elements of the ellipsoids' largest cross-sections (the phantom a
    scanner's geometry is made from)."""
    return [("ellipse", float(e[0]), float(e[1]), float(e[3]), float(e[4]), float(e[6]),
             float(e[7])) for e in np.asarray(ellipsoids).reshape(-1, 8)]
