"""The learned density surrogate's tensor-core kernels against a float64
reference of the same network (torch on the CPU).

Tolerances: the kernels keep weights and activations in BF16 (8-bit
mantissa) and accumulate in FP32, so the forward value and the gradient agree
with float64 to about 1% (relative L2 per parameter block), which these
tests bound at 5%; the reference uses the BF16-rounded hidden weights the
kernels use.
"""
import math

import numpy as np
import pytest

from leven_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

LO, HI = (-1024.0, -128.0, -1024.0), (1024.0, 128.0, 1024.0)
IN = [96, 128, 128, 128]


def unpack(p):
    """Flat parameters -> [(W, b)] x 4 + (w4, b4), float64 tensors."""
    out, o = [], 0
    for k in IN:
        w = torch.tensor(p[o:o + 128 * k], dtype=torch.float64).reshape(128, k)
        o += 128 * k
        b = torch.tensor(p[o:o + 128], dtype=torch.float64)
        o += 128
        out.append((w, b))
    w4 = torch.tensor(p[o:o + 128], dtype=torch.float64)
    b4 = torch.tensor(p[o + 128:o + 129], dtype=torch.float64)
    return out, w4, b4


def bf16(t):
    return t.to(torch.bfloat16).to(torch.float64)


def features(pts):
    cols = []
    for a in range(3):
        ext = HI[a] - LO[a]
        top = math.log2(max(2.0, ext / 2.0))
        u = 2.0 * (torch.tensor(pts[:, a], dtype=torch.float64) - LO[a]) / ext - 1.0
        f = torch.tensor([2.0 ** (top * k / 15) for k in range(16)], dtype=torch.float64)
        ang = math.pi * u[:, None] * f[None, :]
        cols += [torch.sin(ang), torch.cos(ang)]
    return bf16(torch.cat(cols, dim=1))


def reference(p, pts, targets=None, scale=8.0):
    layers, w4, b4 = unpack(p)
    params = [t.clone().requires_grad_(True) for wb in layers for t in wb] + [w4.clone().requires_grad_(True),
                                                                           b4.clone().requires_grad_(True)]
    x = features(pts)
    for i in range(4):
        w, b = params[2 * i], params[2 * i + 1]
        w_eff = w + (bf16(w.detach()) - w.detach())  # the BF16 value, the gradient of w
        x = torch.nn.functional.silu(x @ w_eff.T + b)
    y = x @ params[8] + params[9]
    if targets is None:
        return (y * scale).detach().numpy()
    loss = torch.mean((y - torch.tensor(targets, dtype=torch.float64) / scale) ** 2)
    loss.backward()
    g = np.concatenate([t.grad.numpy().ravel() for t in params])
    return g, loss.item()


@pytest.fixture
def surrogate(lvn_gpu):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    s = lvn.Surrogate(LO, HI, seed=3)
    yield s
    s.close()


def blocks():
    o = 0
    for k in IN:
        yield o, o + 128 * k
        yield o + 128 * k, o + 128 * k + 128
        o += 128 * k + 128
    yield o, o + 128
    yield o + 128, o + 129


def test_forward_matches_float64(surrogate):
    pts = surrogate.sample(1024, seed=5, fetch=True)
    got = surrogate.eval(pts)
    want = reference(surrogate.params(), pts)
    err = np.abs(got - want)
    assert np.linalg.norm(got - want) <= 0.05 * np.linalg.norm(want) + 1e-3, err.max()


@pytest.mark.parametrize("n", [512, 40960])
def test_gradient_matches_float64(surrogate, n):
    """512 rows: one 128-row tile per CTA of the fused training kernel;
    40960 rows (320 tiles): several tiles per CTA, the weight gradients
    accumulated over them in tensor memory, and a last CTA with fewer."""
    pts = surrogate.sample(n, seed=7, fetch=True)
    g, loss = surrogate.grad(pts)
    rg, rloss = reference(surrogate.params(), pts, pts[:, 3])
    assert abs(loss - rloss) <= 0.02 * rloss
    for a, b in blocks():
        num = np.linalg.norm(g[a:b] - rg[a:b])
        assert num <= 0.05 * np.linalg.norm(rg[a:b]) + 1e-7, (a, b, num, np.linalg.norm(rg[a:b]))


def test_training_reduces_loss(surrogate):
    surrogate.sample(1 << 18, seed=11)
    losses = surrogate.train(200, batch=8192, lr=1e-3)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.5 * losses[:5].mean(), (losses[:5], losses[-20:])
    # the trained weights are the ones the kernels evaluate
    pts = surrogate.sample(512, seed=13, fetch=True)
    got = surrogate.eval(pts)
    want = reference(surrogate.params(), pts)
    assert np.linalg.norm(got - want) <= 0.05 * np.linalg.norm(want) + 1e-3


def test_surrogate_meshing_gate(lvn_gpu, surrogate):
    """Chunks take the surrogate's field only where its probe gate passes and
    the chunk lies in its domain; a closed gate gives the plain meshes
    exactly, an open one valid meshes from the surrogate's field."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    surrogate.sample(1 << 18, seed=17)
    surrogate.train(300, batch=8192, lr=1e-3)
    chunks = [((256 * i, 0, 256 * j), 256) for i in range(-2, 2) for j in range(-2, 2)] + [((8192, 0, 0), 256)]
    g = lvn.MeshGen(64)
    try:
        V0, T0, S0, _ = g.generate_chunks(chunks)
        g.set_surrogate(surrogate, gate=0.0)
        V1, T1, S1, _ = g.generate_chunks(chunks)
        assert g.surrogate_chunks(len(chunks)).sum() == 0
        assert np.array_equal(V1.view(np.int32), V0.view(np.int32)) and np.array_equal(T1, T0)
        g.set_surrogate(surrogate, gate=1e9)
        V2, T2, S2, res = g.generate_chunks(chunks)
        use = g.surrogate_chunks(len(chunks))
        assert use[:-1].all() and not use[-1]  # the last chunk is outside the domain
        assert np.isfinite(V2[:, :8]).all()
        for r in res:
            t = T2[r[2]:r[2] + r[3]]
            if t.size:
                assert t.min() >= 0 and t.max() < r[1]
        assert T2.shape[0] > 0.5 * T0.shape[0]
        # the fallback chunk is the plain one
        r0 = res[-1]
        g.set_surrogate(None)
        V3, T3, S3, res3 = g.generate_chunks(chunks[-1:])
        assert np.array_equal(T2[r0[2]:r0[2] + r0[3]], T3)
    finally:
        g.close()


def test_lattice_and_point_evaluation_agree(lvn_gpu, surrogate):
    """The fused inference kernel gives the same densities for a lattice as
    for the same positions passed explicitly."""
    import ctypes as C

    lvn = lvn_gpu
    lat = np.array([[-100.0, -20.0, 37.0, 2.0], [500.0, 3.0, -900.0, 0.5]], np.float32)
    dim = 9
    d_lat = torch.tensor(lat, device="cuda")
    d_out = torch.zeros(2 * dim ** 3, dtype=torch.float32, device="cuda")
    rc = lvn.lib().lvn_surrogate_eval_lattices(surrogate._h, d_lat.data_ptr(), 2, dim, d_out.data_ptr())
    assert rc == 0
    torch.cuda.synchronize()
    pts = []
    for o in lat:
        for k in range(dim):
            for j in range(dim):
                for i in range(dim):
                    pts.append((o[0] + o[3] * i, o[1] + o[3] * j, o[2] + o[3] * k))
    got = surrogate.eval(np.array(pts, np.float32))
    assert np.array_equal(d_out.cpu().numpy().view(np.int32), got.view(np.int32))


@pytest.mark.parametrize("mode", [1, 2])
def test_density_f64_reference(lvn_gpu, mode):
    """The FP64 density agrees with the FP32 restatement of the same density
    (the oracle's) to float rounding: |d32 - d64| <= 1e-4 (1 + |d|)."""
    import ctypes

    import oracle_lib as O

    lvn = lvn_gpu
    dens = W.FBM2D if mode == 1 else W.CAVES
    lvn.set_density(**dens)
    rng = np.random.default_rng(3)
    pts = np.stack([rng.uniform(-2000, 2000, 4096), rng.uniform(-100, 100, 4096), rng.uniform(-2000, 2000, 4096)], 1)
    d64 = lvn.density_f64(pts)
    O.set_seed(1)
    od = O.density(mode=mode)
    d32 = np.array([O.lib().orc_density_at(ctypes.byref(od), *map(float, p)) for p in pts[:256]])
    assert np.abs(d32 - d64[:256]).max() <= 1e-4 * (1 + np.abs(d64[:256]).max())


def test_extrapolation_beyond_the_y_range(surrogate):
    """Above and below the domain's y range the density continues from the
    range's edge with unit slope, so tall coarse chunks keep the sign of
    y - h(x, z) far from the surface."""
    x, z = 123.0, -456.0
    inside = np.array([[x, HI[1], z], [x, LO[1], z]], np.float32)
    outside = np.array([[x, HI[1] + 10.0, z], [x, LO[1] - 7.0, z]], np.float32)
    d_in = surrogate.eval(inside)
    d_out = surrogate.eval(outside)
    assert np.allclose(d_out, d_in + np.array([10.0, -7.0]), rtol=1e-5, atol=1e-4), (d_in, d_out)


def test_trained_network_gain_over_the_method_without_it(lvn_gpu):
    """What the trained network gains.  On held-out samples of the 2D fBm
    density (a 512 x 256 x 512 domain), the trained MLP's density error is set
    against (a) the same network untrained and (b) the method without the
    network: the same 96 Fourier features with the best linear read-out, a
    float64 least-squares fit on the network's own training samples.  The
    trained network must cut the untrained one's RMS error 5-fold and beat the
    linear read-out by 1.5x.  Then, meshing 16 chunks under a probe gate of 8
    voxels (every one of a chunk's 512 probes within 8 density units of the
    plain density), the trained network takes chunks off the plain noise path
    that the untrained one cannot (it falls back everywhere), and the meshes
    it makes index their own vertices."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    lo, hi = (-256.0, -128.0, -256.0), (256.0, 128.0, 256.0)
    s = lvn.Surrogate(lo, hi, seed=7)
    try:
        train = s.sample(1 << 18, seed=21, fetch=True)
        held = s.sample(1 << 14, seed=22, fetch=True)
        s.sample(1 << 18, seed=21)
        rms_untrained = float(np.sqrt(np.mean((s.eval(held) - held[:, 3]) ** 2)))
        g = lvn.MeshGen(64)
        g.set_option(lvn.LVN_OPT_CACHE, 0)
        chunks = [((256 * i, 0, 256 * j), 256) for i in range(-2, 2) for j in range(-2, 2)]
        g.set_surrogate(s, gate=8.0)
        g.generate_chunks(chunks)
        used_untrained = int(g.surrogate_chunks(len(chunks)).sum())
        s.train(3000, batch=16384, lr=1e-3)
        rms_trained = float(np.sqrt(np.mean((s.eval(held) - held[:, 3]) ** 2)))
        V, T, S, res = g.generate_chunks(chunks)
        used_trained = int(g.surrogate_chunks(len(chunks)).sum())
        g.close()
        for r in res:
            t = T[r[2]:r[2] + r[3]]
            assert t.size == 0 or (t.min() >= 0 and t.max() < r[1])
    finally:
        s.close()

    def feats(p):
        cols = []
        for a in range(3):
            ext = hi[a] - lo[a]
            top = math.log2(max(2.0, ext / 2.0))
            u = 2.0 * (p[:, a].astype(np.float64) - lo[a]) / ext - 1.0
            f = 2.0 ** (top * np.arange(16) / 15)
            ang = math.pi * u[:, None] * f[None, :]
            cols += [np.sin(ang), np.cos(ang)]
        return np.concatenate(cols + [np.ones((len(p), 1))], axis=1)

    coef, *_ = np.linalg.lstsq(feats(train), train[:, 3].astype(np.float64), rcond=None)
    rms_linear = float(np.sqrt(np.mean((feats(held) @ coef - held[:, 3]) ** 2)))
    print(f"density RMS error: untrained {rms_untrained:.3f}, linear Fourier read-out {rms_linear:.3f}, "
          f"trained {rms_trained:.3f}; chunks on the surrogate at an 8-voxel gate: {used_untrained} -> {used_trained}")
    assert rms_trained * 5.0 <= rms_untrained, (rms_trained, rms_untrained)
    assert rms_trained * 1.5 <= rms_linear, (rms_trained, rms_linear)
    assert used_untrained == 0 and used_trained > used_untrained
