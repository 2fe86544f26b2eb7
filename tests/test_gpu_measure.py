"""Measurement histograms on the GPU (mdg_measure_*) against the oracle on the same inputs: integer
histograms (ngc, nefipos, ngang, ngz, ng2d1/2) bit-exact, floating-point ones (efipos, tefipos,
ndip*, ftot) to 1e-10 of their scale, for both arithmetic forms of the force phases."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from tests.golden.fixture import y_n_case

pytestmark = pytest.mark.gpu

RDEL = 0.1
INT_KEYS = ("ngc", "nefipos", "ngang", "ngz", "ng2d1", "ng2d2")
FLOAT_KEYS = ("efipos", "tefipos", "ndipx", "ndipy", "ndipz", "ndipsq")
FLOAT_RTOL = 1e-10

CASES = {
    "electrolyte": lambda: configs.slab_electrolyte(),
    "slab": lambda: configs.slab_water(nwat=512, cells=6, placement="lattice"),
    "bulk": lambda: configs.bulk_water(),
    "y_n": lambda: y_n_case()[:2],
}


def _pair(gpulib, oracle, name, precision=abi.MDG_FP64, **kw):
    s, prm = CASES[name]()
    prm = abi.RunParams(**{**prm.__dict__, "precision": precision})
    g = abi.Context(gpulib, s.copy(), prm)
    r = abi.Context(oracle, s.copy(), abi.RunParams(**{**prm.__dict__, "precision": abi.MDG_FP64}))
    dg = g.measure_init(RDEL, **kw)
    dr = r.measure_init(RDEL, **kw)
    assert dg == dr
    return s, g, r


def _compare(hg, hr, float_rtol=FLOAT_RTOL, exact=True):
    for k in INT_KEYS:
        if exact:
            np.testing.assert_array_equal(hg[k], hr[k], err_msg=k)
        else:
            assert hg[k].sum() == hr[k].sum(), k
    for k in FLOAT_KEYS:
        scale = max(np.abs(hr[k]).max(), 1e-30)
        assert np.abs(hg[k] - hr[k]).max() <= float_rtol * scale, (k, np.abs(hg[k] - hr[k]).max() / scale)
    scale = max(np.abs(hr["ftot"]).max(), 1e-30)
    assert np.abs(hg["ftot"] - hr["ftot"]).max() <= float_rtol * scale
    for k in ("calls_force", "calls_do", "out_of_range"):
        assert hg[k] == hr[k], k


@pytest.mark.parametrize("name", list(CASES))
def test_force_histograms(name, gpulib, oracle):
    s, g, r = _pair(gpulib, oracle, name)
    for _ in range(2):  # accumulation over two evaluations
        g.force_get(s.copy())
        r.force_get(s.copy())
    hg, hr = g.measure_get(), r.measure_get()
    assert hr["calls_force"] == 2
    if name == "electrolyte":
        assert hr["nefipos"].sum() == 2 * (s.nliqa - s.nriga) and np.abs(hr["efipos"]).max() > 0
    if name == "y_n":
        assert hr["ngang"].sum() == 2 * 54
    if name in ("slab", "electrolyte", "y_n"):
        assert hr["ngc"].sum() > 0
    _compare(hg, hr)
    g.close()
    r.close()


def test_force_histograms_mixed(gpulib, oracle):
    """The histograms are FP64 side computations: the mixed force form gives the same integer
    histograms; efipos and tefipos carry the mixed forces (ions' fz), so within the mixed
    force tolerance."""
    s, g, r = _pair(gpulib, oracle, "electrolyte", precision=abi.MDG_MIXED)
    g.force_get(s.copy())
    r.force_get(s.copy())
    hg, hr = g.measure_get(), r.measure_get()
    for k in INT_KEYS:
        np.testing.assert_array_equal(hg[k], hr[k], err_msg=k)
    for k in ("efipos", "tefipos"):
        scale = np.abs(hr[k]).max()
        assert np.abs(hg[k] - hr[k]).max() <= 1e-4 * scale, k
    g.close()
    r.close()


def test_measure_do_dropin(gpulib, oracle):
    s, g, r = _pair(gpulib, oracle, "y_n", force_hist=False, l2d=True, rfrst=3.0, rscnd=6.0)
    g.force_get(s.copy())
    r.force_get(s.copy())
    for _ in range(3):
        g.measure_do(s)
        r.measure_do(s)
    hg, hr = g.measure_get(), r.measure_get()
    assert hr["calls_do"] == 3 and hr["ng2d1"].sum() > 0
    _compare(hg, hr)
    g.measure_zero()
    assert g.measure_get()["ngz"].sum() == 0
    g.close()
    r.close()


def test_resident_profiles(gpulib, oracle):
    """Resident steps with force histograms and measure_do after every step: the GPU graph
    against the oracle's step loop."""
    s, g, r = _pair(gpulib, oracle, "electrolyte", force_hist=True, profiles=True, l2d=True, rfrst=3.0,
                    rscnd=6.0)
    g.set_state(s.copy())
    r.set_state(s.copy())
    g.run(4)
    r.run(4)
    hg, hr = g.measure_get(), r.measure_get()
    assert hr["calls_do"] == 4 and hr["calls_force"] == 4
    _compare(hg, hr, float_rtol=1e-8)
    # switching off leaves the arrays as they are
    g.measure_enable(False, False)
    g.run(2)
    assert g.measure_get()["calls_do"] == 4
    g.close()
    r.close()
