"""The bound behind the cave field's shortcut (cave_band in
leven_gb300/csrc/lvn_api.cu): where |y - amp2 h| exceeds |amp3| times a bound
on |fbm3|, the cave term cannot change the sign of the density, so the field
kernel takes the material from the heightfield term alone.

The bound used is |snoise3| <= 1.2972 (simplex.cl:218-289 as the oracle
restates it).  Each of a point's four simplex corners contributes
32 (0.6 - r^2)^4 dot(g, d) with |dot(g, d)| <= |g| r, and the four corners are
among the lattice points within sqrt(0.6) of the point (farther ones give 0),
so 32 |g|max times the largest lattice sum of (0.6 - r^2)^4 r over a cell
bounds |snoise3|.  The lattice sum is maximised over a grid and widened by its
Lipschitz constant times the grid's half-diagonal."""
import ctypes as C

import numpy as np

import oracle_lib as O

G3 = 1.0 / 6.0
BOUND = 1.2972


def lattice(lo, hi):
    r = np.arange(lo, hi + 1)
    L = np.array([(i, j, k) for i in r for j in r for k in r], float)
    return L, L - L.sum(1, keepdims=True) * G3


def cell_points(n):
    g = (np.arange(n) + 0.5) / n
    U = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    return U - U.sum(1, keepdims=True) * G3  # unskewed positions of one skewed cell


def gradient_norm_max():
    # the gradient table's components, as the UNORM8 texel channel reads them:
    # (64 g + 64) / 255 * 4 - 1 for g in {-1, 0, 1}; two of +-1 and one 0 per gradient
    one, zero = (128 / 255) * 4 - 1, (64 / 255) * 4 - 1
    return np.sqrt(2 * max(one * one, 1.0) + zero * zero)


def test_lattice_outside_range_is_out_of_reach():
    Lfull, Lu = lattice(-3, 4)
    outside = ~np.all((Lfull >= -1) & (Lfull <= 2), axis=1)
    P = cell_points(40)
    D = P[:, None, :] - Lu[None, outside, :]
    dmin = np.sqrt((D * D).sum(-1)).min() - np.sqrt(3) / 80  # grid half-diagonal
    assert dmin > np.sqrt(0.6)


def test_snoise3_bound():
    _, Lu = lattice(-1, 2)
    n = 200
    P = cell_points(n)
    best, maxk = 0.0, 0
    for c in range(0, len(P), 1 << 16):
        D = P[c:c + (1 << 16), None, :] - Lu[None, :, :]
        r2 = np.einsum("pld,pld->pl", D, D)
        t = np.clip(0.6 - r2, 0, None)
        best = max(best, float((t ** 4 * np.sqrt(r2)).sum(1).max()))
        maxk = max(maxk, int((r2 < 0.6).sum(1).max()))
    margin = maxk * 0.6 ** 4 * np.sqrt(3) / (2 * n)  # |d/dr (0.6 - r^2)^4 r| <= 0.6^4 per lattice point
    bound = 32 * gradient_norm_max() * (best + margin)
    assert bound <= BOUND, bound


def test_oracle_snoise3_within_bound():
    rng = np.random.default_rng(3)
    pts = rng.uniform(-300.0, 300.0, (20000, 3)).astype(np.float32)
    L = O.lib()
    vals = np.array([L.orc_snoise3(float(x), float(y), float(z)) for x, y, z in pts])
    assert np.abs(vals).max() <= BOUND


def cave_band(amp3, octaves3, gain3):
    """The band the library computes (cave_band in lvn_api.cu): |amp3| times
    the snoise3 bound times the sum of the octave amplitudes, plus 0.1 %."""
    amp, total = np.float32(1.0), 0.0
    for _ in range(octaves3):
        total += abs(float(amp))
        amp = np.float32(amp * np.float32(gain3))
    return abs(amp3) * BOUND * total * 1.001


def test_cave_term_within_band():
    """The oracle's cave term (its density minus the same density without the
    3D term) stays inside the band at random points of the density space."""
    from leven_gb300 import workloads as W

    O.set_seed(1)
    d = W.CAVES
    caves = O.density(mode=2, octaves2=d["octaves2"], freq2=d["freq2"], lac2=d["lacunarity2"], gain2=d["gain2"],
                      amp2=d["amp2"], octaves3=d["octaves3"], freq3=d["freq3"], lac3=d["lacunarity3"],
                      gain3=d["gain3"], amp3=d["amp3"])
    flat = O.density(mode=2, octaves2=d["octaves2"], freq2=d["freq2"], lac2=d["lacunarity2"], gain2=d["gain2"],
                     amp2=d["amp2"], octaves3=d["octaves3"], freq3=d["freq3"], lac3=d["lacunarity3"],
                     gain3=d["gain3"], amp3=0.0)
    band = cave_band(d["amp3"], d["octaves3"], d["gain3"])
    L = O.lib()
    rng = np.random.default_rng(11)
    pts = rng.uniform(-4096.0, 4096.0, (20000, 3)).astype(np.float32)
    worst = 0.0
    for x, y, z in pts:
        a = L.orc_density_at(C.byref(caves), float(x), float(y), float(z))
        b = L.orc_density_at(C.byref(flat), float(x), float(y), float(z))
        worst = max(worst, abs(a - b))
    assert 0.0 < worst <= band, (worst, band)
