"""The CPU oracle, pinned against golden outputs of the reference's own CUDA
kernels (tests/golden/ref_gpu.npz, recorded by make_golden_refgpu.py from
FunctionOnGPU.cu compiled unmodified), and against known-answer properties
of the math (adjointness, constant data, SIRT/MACE identities)."""
from pathlib import Path

import numpy as np
import pytest

import mtr
import oracle
import phantom
from conftest import rel_l2

GOLD = Path(__file__).parent / "golden" / "ref_gpu.npz"


def load_case(d, name):
    vol = mtr.VolumeSize(*[int(v) for v in d[f"{name}/vol"]])
    axes = []
    k = 0
    while f"{name}/axis{k}/data" in d.files:
        axes.append(mtr.AxisData(d[f"{name}/axis{k}/x_coef"], d[f"{name}/axis{k}/y_coef"], d[f"{name}/axis{k}/data"]))
        k += 1
    no, ni, ls, rho = d[f"{name}/params"]
    return vol, axes, int(no), int(ni), float(ls), float(rho)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


CASES = ["single", "two_axis", "oob", "four_axis"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_wbp_matches_reference_kernels(gold, name):
    vol, axes, *_ = load_case(gold, name)
    got = oracle.wbp(oracle.REF_FAITHFUL, axes[0], vol)
    # WBP has no atomics: FP64 sums in the same order -> equal to float rounding
    assert rel_l2(got, gold[f"{name}/wbp0"]) < 1e-6


@pytest.mark.parametrize("name", CASES)
def test_oracle_sirt_matches_reference_kernels(gold, name):
    vol, axes, no, ni, ls, rho = load_case(gold, name)
    x0 = gold[f"{name}/wbp0"]
    got, norms = oracle.sirt(oracle.REF_FAITHFUL, axes[0], vol, x0, ni, ls, norms=True)
    # the reference's float atomics add in an unspecified order
    assert rel_l2(got, gold[f"{name}/sirt0"]) < 1e-5
    np.testing.assert_allclose(norms, gold[f"{name}/sirt0_norms"], rtol=1e-5)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reconstruct_matches_reference_kernels(gold, name):
    vol, axes, no, ni, ls, rho = load_case(gold, name)
    got = oracle.reconstruct(oracle.REF_FAITHFUL, axes, vol, no, ni, ls, rho)
    assert rel_l2(got, gold[f"{name}/recon"]) < 1e-5


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_close_to_reference(gold, name):
    vol, axes, no, ni, ls, rho = load_case(gold, name)
    got = oracle.reconstruct(oracle.FP64, axes, vol, no, ni, ls, rho)
    assert rel_l2(got, gold[f"{name}/recon"]) < 1e-4


def _small():
    vol = mtr.VolumeSize.make(1, 19, -2, 14, 0, 6)
    return vol, phantom.make_case(vol, 24, np.arange(-60, 61, 20.0), [30.0], 4, "gaussian", 0.02, 7,
                                  axis_cls=mtr.AxisData)


def test_adjointness():
    vol, case = _small()
    a = case.axes[0]
    rng = np.random.default_rng(3)
    x = rng.normal(size=vol.shape)
    y = rng.normal(size=a.data.shape)
    s, _ = oracle.forward(oracle.FP64, a, vol, x)
    bs, _ = oracle.backproject(a, vol, y)
    assert abs((s * y).sum() - (x * bs).sum()) < 1e-9 * np.abs(s * y).sum()


def test_constant_projections_give_constant_wbp():
    vol, case = _small()
    a = case.axes[0]
    const = mtr.AxisData(a.x_coef, a.y_coef, np.full_like(a.data, 3.25))
    w = oracle.wbp(oracle.FP64, const, vol)
    _, c = oracle.backproject(a, vol, np.ones(a.data.shape))
    np.testing.assert_allclose(w[c > 0], 3.25, rtol=1e-12)
    assert np.all(w[c == 0] == 0)


def test_constant_volume_normalised_forward_is_constant():
    vol, case = _small()
    a = case.axes[0]
    s, c = oracle.forward(oracle.FP64, a, vol, np.full(vol.shape, 2.5))
    np.testing.assert_allclose(s[c > 0] / c[c > 0], 2.5, rtol=1e-12)


def test_sirt_residual_decreases_on_consistent_data():
    vol, case = _small()
    a = case.axes[0]
    x_true = np.random.default_rng(9).uniform(0, 1, vol.shape)
    s, c = oracle.forward(oracle.FP64, a, vol, x_true)
    b = np.where(c > 0, s / np.where(c > 0, c, 1), 0).astype(np.float32)
    cons = mtr.AxisData(a.x_coef, a.y_coef, b)
    _, norms = oracle.sirt(oracle.FP64, cons, vol, np.zeros(vol.shape), 12, 0.5, norms=True)
    assert np.all(np.diff(norms) < 0)


def test_single_axis_mace_half_step_is_sirt():
    vol, case = _small()
    a = case.axes[0]
    # z = w, so w <- 0.5(2v - w) + 0.5w = v up to the rounding of the update
    for mode, tol in ((oracle.REF_FAITHFUL, 1e-6), (oracle.FP64, 1e-14)):
        x0 = oracle.wbp(mode, a, vol)
        want = oracle.sirt(mode, a, vol, x0, 10, 0.5)
        got = oracle.reconstruct(mode, [a], vol, 1, 10, 0.5, 0.5)
        assert rel_l2(got, want) < tol


def test_identical_axes_consensus():
    # K identical axes: every w_k stays equal, so w_avg == w_k.
    vol, case = _small()
    a = case.axes[0]
    out, w = oracle.reconstruct(oracle.FP64, [a, a, a], vol, 2, 3, 0.5, 0.7, with_axes=True)
    np.testing.assert_allclose(w[0], w[1], rtol=0, atol=0)
    np.testing.assert_allclose(out, w[0], rtol=1e-12, atol=1e-12)


def test_ref_faithful_close_to_fp64():
    vol, case = _small()
    r0 = oracle.reconstruct(oracle.REF_FAITHFUL, case.axes, vol, 2, 4, 0.5, 0.7)
    r1 = oracle.reconstruct(oracle.FP64, case.axes, vol, 2, 4, 0.5, 0.7)
    assert rel_l2(r0, r1) < 1e-5


@pytest.mark.parametrize("myid,n,z,s,want", [(0, 4, 10, 0, (0, 3)), (1, 4, 10, 0, (3, 6)), (2, 4, 10, 0, (6, 8)),
                                             (3, 4, 10, 0, (8, 10)), (0, 1, 7, -3, (-3, 4)), (2, 3, 9, 5, (11, 14))])
def test_divide_slice(myid, n, z, s, want):
    # MultiAxis.cpp:13-31: the first Z % N slabs get one extra section
    assert oracle.divide_slice(myid, n, z, s) == want


def test_thread_count_does_not_change_results():
    vol, case = _small()
    n = oracle.num_threads()
    oracle.set_threads(1)
    r1 = oracle.reconstruct(oracle.REF_FAITHFUL, case.axes, vol, 1, 3, 0.5, 0.7)
    oracle.set_threads(max(2, n))
    r2 = oracle.reconstruct(oracle.REF_FAITHFUL, case.axes, vol, 1, 3, 0.5, 0.7)
    oracle.set_threads(n)
    np.testing.assert_array_equal(r1, r2)
