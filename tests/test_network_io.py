"""Network-parameter post-processing and the Touchstone writer (host code
behind the C-ABI, no GPU): the known-answer cases of the reference's
tests/test_coupling.cpp and tests/test_touchstone_nport.cpp, and parity with
the oracle on seeded random S matrices (text byte for byte, matrices to
rounding)."""
import math

import numpy as np
import pytest

import edgefem_oracle as O

import edgefem_gb300 as em
from edgefem_gb300 import _lib


def rand_S(rng, n, scale=0.4):
    return scale * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / math.sqrt(n)


# ---------------------------------------------- tests/test_coupling.cpp cases

def test_coupling_known_answers():
    cm = em.compute_coupling(np.zeros((2, 2)), 10e9, 50.0)             # :11-28
    assert cm.num_ports == 2 and cm.z0 == 50.0 and cm.frequency == 10e9
    assert np.allclose(cm.Z, 50.0 * np.eye(2), rtol=0, atol=1e-10 * 50)
    assert abs(em.compute_coupling([[-1.0]], 10e9, 50.0).Z[0, 0]) < 1e-10  # :30-43 short circuit
    S = np.array([[0.1, 0.01, 0.001], [0.01, 0.1, 0.01], [0.001, 0.01, 0.1]])  # :45-71
    db = em.mutual_coupling_db(em.compute_coupling(S, 10e9))
    assert abs(db[0, 0] - 20 * math.log10(0.1)) < 0.1 and abs(db[0, 1] - 20 * math.log10(0.01)) < 0.1
    S2 = np.array([[0.1, 0.3], [0.3, 0.1]])                              # :73-110
    assert abs(em.active_reflection(S2, [1, 1])[0] - 0.4) < 1e-10
    assert abs(em.active_reflection(S2, [1, -1])[0] + 0.2) < 1e-10
    assert not em.is_passive([[0, 2], [2, 0]])                           # :128-139
    a = 1 / math.sqrt(2)                                                 # :141-161
    assert not em.is_lossless([[0, 1j * a], [1j * a, 0]], 1e-6)
    assert em.is_lossless([[0, 1j], [1j, 0]], 1e-6)
    assert em.is_reciprocal([[0.1 + 0.1j, 0.9], [0.9, 0.1 + 0.1j]])      # :163-180
    assert not em.is_reciprocal([[0, 0], [1, 0]], 1e-6)


def test_is_passive_follows_the_singular_value_rule():
    """tests/test_coupling.cpp:114-126 asserts is_passive for j[[0.3, 0.9],
    [0.9, 0.3]], reasoning from the column power sum 0.9; its singular values
    are 1.2 and 0.6, so the rule of src/coupling.cpp:96-112 (every singular
    value <= 1 + tol) says not passive.  Both here and in the oracle the rule
    decides."""
    S = np.array([[0.3j, 0.9j], [0.9j, 0.3j]])
    assert np.allclose(em.singular_values(S), [1.2, 0.6], rtol=1e-14)
    assert em.is_passive(S) is False and O.is_passive(S) is False
    assert em.is_passive(0.8 * S / 1.2) and em.check_passivity(0.8 * S / 1.2)


def test_coupling_matches_oracle():
    rng = np.random.default_rng(7)
    for n in (1, 2, 3, 5, 8):
        for _ in range(4):
            S = rand_S(rng, n)
            cm = em.compute_coupling(S, 5e9, 75.0)
            Z, Y = O.compute_coupling(S, 75.0)
            assert np.abs(cm.Z - Z).max() <= 1e-11 * np.abs(Z).max()
            assert np.abs(cm.Y - Y).max() <= 1e-11 * np.abs(Y).max()
            assert np.allclose(em.singular_values(S), np.linalg.svd(S, compute_uv=False), rtol=1e-12, atol=1e-14)
            for tol in (1e-6, 1e-2):
                assert em.is_passive(S, tol) == O.is_passive(S, tol)
                assert em.is_reciprocal(S, tol) == O.is_reciprocal(S, tol)
                assert em.is_lossless(S, tol) == O.is_lossless(S, tol)
            a = rng.normal(size=n) + 1j * rng.normal(size=n)
            assert np.allclose(em.active_reflection(S, a), O.active_reflection(S, a), rtol=1e-13, atol=1e-15)
            assert np.allclose(em.mutual_coupling_db(cm), O.mutual_coupling_db(S), rtol=1e-14, atol=0)
    # a unitary, symmetric S: lossless and reciprocal; passive at the boundary
    Q = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0]
    U = Q @ Q.T
    assert em.is_lossless(U) and em.is_reciprocal(U) and em.is_passive(U)


def test_coupling_singular_factor_is_regularised():
    """S = I makes I - S singular (open circuit): the reference adds 1e-12 I."""
    cm = em.compute_coupling(np.eye(2), 1e9, 50.0)
    Z, Y = O.compute_coupling(np.eye(2), 50.0)
    assert np.allclose(cm.Z, Z, rtol=1e-12) and np.allclose(cm.Y, Y, atol=1e-20)
    assert abs(cm.Z[0, 0] - 50.0 * 2 / 1e-12) <= 1e-6 * abs(cm.Z[0, 0])


def test_coupling_rejects_bad_input():
    with pytest.raises(ValueError, match="square"):
        em.compute_coupling(np.zeros((2, 3)), 1e9)
    with pytest.raises(ValueError, match="Excitation"):
        em.active_reflection(np.zeros((2, 2)), [1, 2, 3])
    assert em.is_passive(np.zeros((2, 3))) is False


# ------------------------------------------ tests/test_touchstone_nport.cpp

def test_touchstone_extension():
    for n, e in ((1, ".s1p"), (2, ".s2p"), (3, ".s3p"), (4, ".s4p"), (10, ".s10p")):
        assert em.touchstone_extension(n) == e
    for bad in (0, 100):
        with pytest.raises(_lib.EdgefemError, match="Invalid number of ports"):
            em.touchstone_extension(bad)


@pytest.mark.parametrize("fmt,name", [(0, "RI"), (1, "MA"), (2, "DB")])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_touchstone_nport_text_matches_oracle(tmp_path, fmt, name, n):
    rng = np.random.default_rng(100 + n)
    freqs = [1e9, 2.5e9, 3.125e9, 12e9]
    S = [rand_S(rng, n) for _ in freqs]
    S[0][0, 0] = 0.0           # |S| clamped at 1e-20 in dB form
    S[1][0, 0] = -0.2 + 0.0j   # angle at +180
    path = tmp_path / f"x{em.touchstone_extension(n)}"
    em.write_touchstone_nport(str(path), freqs, S, em.TouchstoneOptions(fmt, 50.0))
    assert path.read_text() == O.touchstone_nport_text(freqs, S, name, 50.0)


def test_touchstone_reference_headers(tmp_path):
    """test_touchstone_nport.cpp:25-138: the option line of each format."""
    S3 = np.array([[0.1, -0.3 + 0.1j, -0.2], [-0.3 + 0.1j, 0.1, -0.3 + 0.1j], [-0.2, -0.3 + 0.1j, 0.1]])
    S4 = np.full((4, 4), -0.2 + 0.05j)
    np.fill_diagonal(S4, 0.1)
    S2 = np.array([[0.1, -0.9 + 0.1j], [-0.9 + 0.1j, 0.1]])
    for fmt, S, freqs, opt in ((0, S3, [1e9, 2e9, 3e9], "Hz S RI R 50"), (1, S4, [1e9, 2e9], "Hz S MA R 50"),
                               (2, S2, [1e9], "Hz S DB R 50")):
        p = tmp_path / f"t{S.shape[0]}.s{S.shape[0]}p"
        em.write_touchstone_nport(str(p), freqs, [S] * len(freqs), em.TouchstoneOptions(fmt, 50.0))
        lines = p.read_text().splitlines()
        assert opt in lines[2]
    # a 4-port frequency spans 4 lines of 4 values; continuation lines carry no frequency
    body = (tmp_path / "t4.s4p").read_text().splitlines()[3:]
    assert len(body) == 8 and body[0].startswith("1000000000 ") and body[1].startswith(" ")


def test_touchstone_errors(tmp_path):
    with pytest.raises(_lib.EdgefemError, match="Empty"):
        em.write_touchstone_nport(str(tmp_path / "e.s2p"), [], [])
    with pytest.raises(_lib.EdgefemError, match="mismatch"):
        em.write_touchstone_nport(str(tmp_path / "m.s2p"), [1e9, 2e9, 3e9], [np.array([[0.1, -0.9], [-0.9, 0.1]])])
    with pytest.raises(_lib.EdgefemError, match="Cannot open"):
        em.write_touchstone_nport(str(tmp_path / "no_dir" / "x.s2p"), [1e9], [np.eye(2)])


def test_touchstone_legacy_2port(tmp_path):
    rng = np.random.default_rng(3)
    freqs = [8e9, 9e9, 10e9]
    S = [rand_S(rng, 2) for _ in freqs]
    p = tmp_path / "legacy.s2p"
    em.write_touchstone(str(p), freqs, S)
    assert p.read_text() == O.touchstone_2port_text(freqs, S)


def test_design_export_touchstone(tmp_path):
    """RectWaveguideDesign.export_touchstone (waveguide.py:436-464) with given data."""
    wg = em.RectWaveguideDesign(a=22.86e-3, b=10.16e-3, length=50e-3)
    with pytest.raises(RuntimeError, match="No simulation data"):
        wg.export_touchstone(str(tmp_path / "none"))
    S = [np.array([[0.1, 0.9j], [0.9j, 0.1]])]
    wg.export_touchstone(str(tmp_path / "wg"), [10e9], S)
    assert (tmp_path / "wg.s2p").read_text() == O.touchstone_nport_text([10e9], S, "RI", 50.0)
