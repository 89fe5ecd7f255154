"""Shared helpers for the GPU parity tests: one cluster description feeds both
the oracle and the GPU library."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
nm = 1e-9


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def oracle_cluster(O, g):
    chi = g["chi"] if "chi" in g.files else np.zeros(3, np.complex128)
    return O.Cluster(xyz=g["xyz"], radius=g["radius"], eps=g["eps"], mu=g["mu"], eps_sh=g["eps_sh"],
                     nmax=int(g["nmax"]), wavelength=float(g["wavelength"]),
                     bg_eps=complex(g["bg"][0]), bg_mu=complex(g["bg"][1]),
                     theta=float(g["angles"][0]), phi=float(g["angles"][1]),
                     e_theta=complex(g["pol"][0]), e_phi=complex(g["pol"][1]),
                     ksippp=complex(chi[0]), ksiparppar=complex(chi[1]), gamma=complex(chi[2]))


def gpu_inputs(G, cl):
    """(spheres, medium, wave) for the GPU library from an oracle Cluster."""
    sp = G.spheres_array(cl.xyz, cl.radius, cl.eps, cl.nmax, mu=cl.mu, eps_sh=cl.eps_sh,
                         ksippp=cl.chi[:, 0], ksiparppar=cl.chi[:, 1], gamma=cl.chi[:, 2])
    return sp, G.medium(cl.bg_eps, cl.bg_mu), G.plane_wave(cl.wavelength, cl.theta, cl.phi,
                                                           cl.e_theta, cl.e_phi)


def random_cluster(rng, n, edge, rmin, rmax, gap):
    """Seeded rejection sampling of non-overlapping spheres in a cube of side
    `edge` centred on the origin; radii uniform in [rmin, rmax]; gap >= `gap`."""
    xyz, rad = [], []
    tries = 0
    while len(xyz) < n:
        tries += 1
        if tries > 200000:
            raise RuntimeError("cannot place spheres")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(-edge / 2 + r, edge / 2 - r, size=3)
        if xyz:
            d = np.linalg.norm(np.array(xyz) - c, axis=1) - np.array(rad) - r
            if d.min() < gap:
                continue
        xyz.append(c)
        rad.append(r)
    return np.array(xyz), np.array(rad)
