"""Seeded synthetic water/ion systems with the shapes of the benchmark workloads.

Rigid 3-site waters: O on a jittered simple-cubic lattice (uniform +-0.05 nm
per axis), two H at 0.1 nm with a 109.47 degree HOH angle in a uniformly random
orientation (random unit quaternion).  Charges O -0.8476 e, H +0.4238 e (the
SPC/E charges of the reference's exp/settings/*/spce_noexcl.itp, with no
exclusions), Na +1 e, Cl -1 e.  Ions replace whole waters at their O site.
Everything is wrapped into the box.  numpy's PCG64 generator makes the output
identical on every platform for a given seed.

Lattice sites: n_side = ceil(cbrt(n_sites)) per axis with spacing L/n_side; when
n_sites is not a cube the occupied sites are a seeded sample without replacement.
"""
import math

import numpy as np

Q_O = -0.8476
Q_H = 0.4238
Q_NA = 1.0
Q_CL = -1.0
R_OH = 0.1
HOH_DEG = 109.47
# 0.15 mol/L in ion pairs per nm^3
NACL_015M_PER_NM3 = 0.15 * 6.02214076e23 / 1e24


def _random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def water_ion_box(n_sites, box, n_na=0, n_cl=0, seed=0, jitter=0.05, fill_z=1.0):
    """Return (xyz float32 (n,3), q float32 (n,), box float64 (3,)).

    n_sites lattice sites are filled inside [0, box) x [0, box) x [0, fill_z*box_z);
    n_na + n_cl of them (chosen by the seed) hold ions instead of waters.
    Atom order: waters (O, H, H) in site order, then Na, then Cl.
    """
    box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).copy()
    rng = np.random.default_rng(seed)
    ext = box.copy()
    ext[2] *= fill_z
    # lattice with near-cubic spacing over the filled region
    vol = ext.prod()
    a = (vol / n_sites) ** (1.0 / 3.0)
    ns = np.maximum(1, np.ceil(ext / a - 1e-9)).astype(int)
    while ns.prod() < n_sites:
        ns[np.argmin(ext / ns)] += 0  # keep spacing near-isotropic
        ns[np.argmax(ext / ns)] += 1
    sp = ext / ns
    total = int(ns.prod())
    pick = np.sort(rng.choice(total, size=n_sites, replace=False)) if total > n_sites else np.arange(total)
    iz = pick % ns[2]
    iy = (pick // ns[2]) % ns[1]
    ix = pick // (ns[2] * ns[1])
    sites = (np.stack([ix, iy, iz], 1) + 0.5) * sp
    sites += rng.uniform(-jitter, jitter, size=sites.shape)
    n_ion = n_na + n_cl
    if n_ion > n_sites:
        raise ValueError("more ions than lattice sites")
    ion_slots = rng.choice(n_sites, size=n_ion, replace=False) if n_ion else np.zeros(0, int)
    is_ion = np.zeros(n_sites, bool)
    is_ion[ion_slots] = True
    wsites = sites[~is_ion]
    half = math.radians(HOH_DEG) / 2
    local = np.array([[math.sin(half), 0.0, math.cos(half)], [-math.sin(half), 0.0, math.cos(half)]]) * R_OH
    rot = _random_rotations(rng, len(wsites))
    h = np.einsum("nij,kj->nki", rot, local) + wsites[:, None, :]
    water = np.concatenate([wsites[:, None, :], h], 1).reshape(-1, 3)
    ions = sites[ion_slots]
    xyz = np.concatenate([water, ions[:n_na], ions[n_na:]], 0)
    q = np.concatenate([np.tile([Q_O, Q_H, Q_H], len(wsites)), np.full(n_na, Q_NA), np.full(n_cl, Q_CL)])
    xyz = np.mod(xyz, box)
    xyz32 = xyz.astype(np.float32)
    # float rounding can land exactly on the upper edge; keep every coordinate in [0, box)
    for d in range(3):
        bad = xyz32[:, d] >= np.float32(box[d])
        xyz32[bad, d] = np.float32(0.0)
    return xyz32, q.astype(np.float32), box


def cfg_small():
    """3,000 waters (9,000 atoms) in a 4.5 nm cube; p=8, depth 3."""
    return water_ion_box(3000, 4.5, seed=1)


def cfg_96k():
    """32,000 lattice sites in a 9.86 nm cube, 100 Na+ and 100 Cl- replacing waters
    (31,800 waters + 200 ions = 95,600 atoms); p=10, depth 4."""
    return water_ion_box(32000, 9.86, n_na=100, n_cl=100, seed=2)


def cfg_250k():
    """13.6 nm cube, 83,182 waters + 228 Na+ + 228 Cl- = 250,002 atoms (0.15 M)."""
    return water_ion_box(83182 + 456, 13.6, n_na=228, n_cl=228, seed=5)


def cfg_1m():
    """The large water slab: 333,402 waters + 898 Na+ + 898 Cl- (0.15 M) = 1,002,002
    atoms filling a 21.5 nm cube, depth 5 (30.6 bodies per leaf).  The slab is
    described on a 21.5 x 21.5 x 43 nm box with the upper half empty; the reference's
    solver takes box[XX][XX] as the period of a cube (zeta_fmm_solver.cpp:38-40), so
    the system it solves is this cube, and so does this library (cubic boxes only)."""
    return water_ion_box(333402 + 1796, 21.5, n_na=898, n_cl=898, seed=3)


def cfg_slab_1m():
    """The inhomogeneous 1,002,002-atom system: a periodic 21.5 x 21.5 x 43 nm box
    whose lower half is water (333,402 waters) with 0.15 M NaCl (898 Na+ and 898
    Cl-, about 0.0903 pairs per nm^3 of water) placed uniformly in the water, and
    whose upper half is vacuum."""
    return water_ion_box(333402 + 1796, [21.5, 21.5, 43.0], n_na=898, n_cl=898, seed=3, fill_z=0.5)


def kicked_frames(xyz, box, n_frames, sigma=0.01, seed=7):
    """Frames of a trajectory: each frame adds Gaussian kicks of sigma nm to the
    previous one (wrapped into the box).  Yields float32 coordinates."""
    rng = np.random.default_rng(seed)
    L = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    x = xyz.astype(np.float64)
    for _ in range(n_frames):
        x = np.mod(x + rng.normal(0.0, sigma, size=x.shape), L)
        x32 = x.astype(np.float32)
        for d in range(3):
            x32[x32[:, d] >= np.float32(L[d]), d] = np.float32(0.0)
        yield x32


def batch_systems(n_sys=64, seed=4, nmin=2000, nmax=200000, density=100.2):
    """Independent cubic water+ion boxes, atom counts log-uniform in [nmin, nmax],
    L = (N/density)^(1/3), 0.15 M NaCl.  Returns a list of (xyz, q, box)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_sys):
        n_atoms = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        L = (n_atoms / density) ** (1.0 / 3.0)
        pairs = int(round(NACL_015M_PER_NM3 * L ** 3))
        # sites: waters*3 + ions = n_atoms as closely as possible
        n_sites = (n_atoms - 2 * pairs) // 3 + 2 * pairs
        out.append(water_ion_box(n_sites, L, n_na=pairs, n_cl=pairs, seed=seed * 1000 + k))
    return out
