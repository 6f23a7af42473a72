"""Particle-particle Coulomb sums of the FMM handlers (direct, on the GPU).

Pinned to the reference's own pair kernel with the 1 nm cutoff
(include/ParticleHandler/FMM/FP2PRCutoff.hpp), compiled by the harness with
stand-ins for the few scalFMM names it uses: 256 particles, every target
summed over every other particle in index order, and MutualParticles on
consecutive pairs (tests/golden/p2p_cutoff.npz).

* CPU: the oracle's restatement gives the reference's bits;
* GPU: the engine's FP64 sums within 1e-12 of the oracle (the order of the
  sum differs), FP32 within 1e-4 of the largest force (float positions set
  the error of the nearest pairs); cutoff, self-exclusion, periodic images,
  empty and single-particle inputs, and argument checks.
"""
import numpy as np
import pytest

from conftest import golden

G = "p2p_cutoff.npz"


def _pos(g):
    return np.stack([g["x"], g["y"], g["z"]])


def test_oracle_matches_reference_sums(oracle):
    g = golden(G)
    f, p = oracle.p2p_coulomb(_pos(g), g["q"], 1e9)
    assert np.array_equal(f[0], g["fx"]) and np.array_equal(f[1], g["fy"])
    assert np.array_equal(f[2], g["fz"]) and np.array_equal(p, g["pot"])


def test_oracle_pair_matches_reference_mutual(oracle):
    """MutualParticles gives the target the pair term and the source its
    negative force and its own potential term."""
    g = golden(G)
    pos, q = _pos(g), g["q"]
    m = g["mutual"].reshape(-1, 8)
    for k in range(m.shape[0]):
        a, b = 2 * k, 2 * k + 1
        o = oracle.p2p_pair(pos[:, a], q[a], pos[:, b], q[b])
        r = oracle.p2p_pair(pos[:, b], q[b], pos[:, a], q[a])
        assert np.array_equal(o[:3], m[k, :3]) and o[3] == m[k, 3]
        assert np.array_equal(-o[:3], m[k, 4:7]) and r[3] == m[k, 7]


def test_fixture_has_pairs_inside_the_cutoff():
    g = golden(G)
    pos = _pos(g)
    d = np.linalg.norm(pos[:, 1::7] - pos[:, 0:-1:7][:, :pos[:, 1::7].shape[1]], axis=0)
    assert np.any(d < 1e-9)


def test_oracle_images_sum_the_copies(oracle):
    """One shell of periodic copies: the same as the isolated sum over a
    27-fold replicated set of sources, for the central targets."""
    rs = np.random.default_rng(3)
    n, box = 20, 4e-8
    pos = rs.random((3, n)) * box
    q = np.where(rs.random(n) < 0.5, -1.0, 1.0) * 1.602e-19
    f1, p1 = oracle.p2p_coulomb(pos, q, 1e9, box, 1)
    reps = [pos + np.array([a, b, c])[:, None] * box
            for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)]
    order = [13] + [k for k in range(27) if k != 13]  # central copy first
    big = np.concatenate([reps[k] for k in order], axis=1)
    f2, p2 = oracle.p2p_coulomb(big, np.tile(q, 27), 1e9)
    assert np.allclose(f1, f2[:, :n], rtol=1e-12, atol=1e-12 * np.abs(f2).max())
    assert np.allclose(p1, p2[:n], rtol=1e-12)


# ---- GPU ---------------------------------------------------------------------

def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-4)])
def test_gpu_matches_reference_sums(engine, precision, tol):
    from viennaemc_gb300 import p2p
    g = golden(G)
    f, p = p2p.coulomb(_pos(g), g["q"], 1e9, precision=precision)
    ref_f = np.stack([g["fx"], g["fy"], g["fz"]])
    assert _rel(f, ref_f) <= tol, _rel(f, ref_f)
    assert _rel(p, g["pot"]) <= tol, _rel(p, g["pot"])


@pytest.mark.gpu
@pytest.mark.parametrize("n,images", [(1000, 0), (3000, 0), (300, 1), (257, 2)])
def test_gpu_matches_oracle(engine, oracle, n, images):
    """Sizes off the tile width, the cutoff active, charges of both signs,
    periodic copies."""
    from viennaemc_gb300 import p2p
    rs = np.random.default_rng(n + images)
    box = 1e-7
    pos = rs.random((3, n)) * box
    pos[:, 1::9] = pos[:, 0:-1:9][:, :pos[:, 1::9].shape[1]] + 2e-10  # inside 1 nm
    q = np.where(rs.random(n) < 0.3, 1.0, -1.0) * 1.60219e-19
    fo, po_ = oracle.p2p_coulomb(pos, q, 1e9, box, images)
    f64, p64 = p2p.coulomb(pos, q, 1e9, box, images, "fp64")
    assert _rel(f64, fo) <= 1e-12 and _rel(p64, po_) <= 1e-12
    f32, p32 = p2p.coulomb(pos, q, 1e9, box, images, "fp32")
    assert _rel(f32, fo) <= 5e-5 and _rel(p32, po_) <= 5e-5


@pytest.mark.gpu
def test_gpu_no_cutoff_and_edge_cases(engine, oracle):
    from viennaemc_gb300 import p2p, _lib
    rs = np.random.default_rng(9)
    pos = rs.random((3, 50)) * 1e-8
    q = np.full(50, -1.60219e-19)
    fo, po_ = oracle.p2p_coulomb(pos, q, 0.0)
    f, p = p2p.coulomb(pos, q, 0.0)
    assert _rel(f, fo) <= 1e-12 and _rel(p, po_) <= 1e-12
    # one particle: nothing acts on it; none: nothing to do
    f1, p1 = p2p.coulomb(pos[:, :1], q[:1])
    assert np.all(f1 == 0) and p1[0] == 0
    f0, p0 = p2p.coulomb(np.zeros((3, 0)), np.zeros(0))
    assert f0.shape == (3, 0) and p0.shape == (0,)
    # two like charges repel: the force on the left one points left
    two = np.array([[0.0, 2e-9], [0.0, 0.0], [0.0, 0.0]])
    ft = p2p.force_on_particles(two, np.array([-1.6e-19, -1.6e-19]), 11.7)
    assert ft[0, 0] < 0 < ft[0, 1]
    with pytest.raises(_lib.EmcgError):
        p2p.coulomb(pos, q, 1e9, box=0.0, images=1)
    with pytest.raises(_lib.EmcgError):
        p2p.coulomb(pos, q, -1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-3)])
def test_gpu_cutoff_radius_reference_kat(engine, precision, tol):
    """The reference's cutoff test (tests/testCutOffRadius/testCutOffRadius.cpp:
    46-116): two unit charges 0.17, 0.52 and 5.4 nm apart; below 1 nm the
    distance is taken as 1 nm along the same direction.  Potential q / r and
    force magnitudes |q^2 d / r^3| per component on both particles (1e-10
    relative in FP64; float positions in FP32)."""
    from viennaemc_gb300 import p2p
    a = np.array([50e-9, 50e-9, 50e-9])
    for b in ([50.1e-9, 50.1e-9, 50.1e-9], [50.5e-9, 50.1e-9, 50.1e-9],
              [52e-9, 53e-9, 54e-9]):
        b = np.array(b)
        f, p = p2p.coulomb(np.stack([a, b], axis=1), np.ones(2), 1e9, precision=precision)
        d = a - b
        r = np.linalg.norm(d)
        if r < 1e-9:
            d, r = d * (1e-9 / r), 1e-9
        exp_f, exp_p = np.abs(d) / r ** 3, 1.0 / r
        for i in range(2):
            assert abs(p[i] - exp_p) <= tol * exp_p, (b, i, p[i], exp_p)
            assert np.allclose(np.abs(f[:, i]), exp_f, rtol=tol, atol=0), (b, i, f[:, i], exp_f)
