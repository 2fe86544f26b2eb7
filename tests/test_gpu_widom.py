"""Widom insertion on the GPU (mdg_widom) against the oracle's chempot on the same force
evaluation: positions tried, generator state and inave exact; pave to 1e-9 of its largest bin
(FP64 context), 1e-4 with the mixed force form (S(k) from the tensor-core sum)."""
import numpy as np
import pytest

from md_sim_gb300 import abi, configs

pytestmark = pytest.mark.gpu

SEED0 = 14135621772.0


def _pair(gpulib, oracle, precision, nwat=64):
    s, prm = configs.slab_water(nwat=nwat, cells=6, placement="lattice", kmax=6)
    pg = abi.RunParams(**{**prm.__dict__, "precision": precision})
    g = abi.Context(gpulib, s.copy(), pg)
    r = abi.Context(oracle, s.copy(), prm)
    g.force_get(s.copy())
    r.force_get(s.copy())
    return g, r


@pytest.mark.parametrize("flags", [0, abi.MDG_WIDOM_SKIP_OVERLAP, abi.MDG_WIDOM_SKIP_OVERLAP | abi.MDG_WIDOM_EW3DC])
def test_widom_fp64(flags, gpulib, oracle):
    g, r = _pair(gpulib, oracle, abi.MDG_FP64)
    a = g.widom(60, 1.0, 5.0, 8, 4, SEED0, flags=flags)
    b = r.widom(60, 1.0, 5.0, 8, 4, SEED0, flags=flags)
    assert a["done"] == b["done"] and a["seed"] == b["seed"]
    np.testing.assert_array_equal(a["inave"], b["inave"])
    scale = max(b["pave"].max(), 1e-300)
    assert np.abs(a["pave"] - b["pave"]).max() <= 1e-9 * scale, (a["pave"], b["pave"])
    if flags & abi.MDG_WIDOM_SKIP_OVERLAP:
        assert b["done"] == 60 and b["pave"].max() > 0.0
    g.close()
    r.close()


def test_widom_mixed(gpulib, oracle):
    g, r = _pair(gpulib, oracle, abi.MDG_MIXED)
    f = abi.MDG_WIDOM_SKIP_OVERLAP
    a = g.widom(60, 1.0, 5.0, 8, 4, SEED0, flags=f)
    b = r.widom(60, 1.0, 5.0, 8, 4, SEED0, flags=f)
    np.testing.assert_array_equal(a["inave"], b["inave"])
    rel = np.abs(a["pave"] - b["pave"]) / np.maximum(b["pave"], 1e-300)
    assert np.all(rel[b["pave"] > 1e-12 * b["pave"].max()] <= 1e-4), rel
    g.close()
    r.close()


def test_widom_dense_stops_at_first_overlap(gpulib, oracle):
    g, r = _pair(gpulib, oracle, abi.MDG_FP64, nwat=512)
    a = g.widom(200, 2.0, 6.0, 8, 4, SEED0)
    b = r.widom(200, 2.0, 6.0, 8, 4, SEED0)
    assert a["done"] == b["done"] < 200
    assert a["seed"] == b["seed"]
    np.testing.assert_array_equal(a["inave"], b["inave"])
    g.close()
    r.close()
