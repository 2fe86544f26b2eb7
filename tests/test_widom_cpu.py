"""Widom insertion (chempot, src/forcem.f90:1226-1507) in the oracle: the reference's generator
(src/rndmod.f90:26-35) restated independently here, the generator state after a call, the
reference's stop at the first overlapping position, and the accumulation of pave/inave."""
import numpy as np

from md_sim_gb300 import abi, configs

SEED0 = 14135621769.0 + 3.0   # rnd_init of rank 0 (src/measure.f90:149)


def rnd(state):
    state[0] = np.fmod(8192.0 * state[0], 67099547.0)
    return state[0] * 1.4903230270690e-8


def _ctx(lib, nwat=64):
    s, prm = configs.slab_water(nwat=nwat, cells=6, placement="lattice", kmax=6)
    c = abi.Context(lib, s.copy(), prm)
    c.force_get(s.copy())
    return s, c


def test_generator_state_after_first_position(oracle):
    s, c = _ctx(oracle, nwat=128)
    lwmin, lwmax = 1.0, 5.0
    r = c.widom(40, lwmin, lwmax, 8, 4, SEED0)
    assert r["done"] >= 1
    # replay: positions are drawn (x, y, then z until |z| > the inner bound), orientations only
    # for accepted positions; the call ends at the first overlap
    st = [SEED0]
    zlo, zhi = s.lwh - lwmax, s.lwh - lwmin
    for k in range(r["done"]):
        rnd(st)
        rnd(st)
        while True:
            z = (rnd(st) - 0.5) * zhi * 2.0
            if abs(z) > zlo:
                break
        if k == r["done"] - 1:
            break
        il = int((abs(z) - zlo) * (1.0 / (zhi - zlo) * 8.0)) + 1
        for _ in range(20 if il > 4 else 1):
            while True:
                h = [rnd(st) - 0.5 for _ in range(3)]
                ri = h[0] * h[0] + h[1] * h[1] + h[2] * h[2]
                if ri < 0.25 and ri > float(np.float32(0.001)):
                    break
            rnd(st)
    assert r["seed"] == st[0]
    c.close()


def test_accumulation_and_determinism(oracle):
    s, c = _ctx(oracle)
    a = c.widom(40, 1.0, 5.0, 8, 4, SEED0, flags=abi.MDG_WIDOM_SKIP_OVERLAP)
    b = c.widom(40, 1.0, 5.0, 8, 4, SEED0, flags=abi.MDG_WIDOM_SKIP_OVERLAP)
    assert a["done"] == 40 and a["seed"] == b["seed"]
    np.testing.assert_array_equal(a["pave"], b["pave"])
    np.testing.assert_array_equal(a["inave"], b["inave"])
    # every position counts 20 orientations above bin 4, one below
    assert a["inave"][:4].sum() + a["inave"][4:].sum() // 20 == 40
    assert np.all(a["inave"][4:] % 20 == 0)
    assert a["pave"].max() > 0.0
    # accumulation into the caller's arrays, generator continued from the returned state
    p, n = a["pave"].copy(), a["inave"].copy()
    c2 = c.widom(10, 1.0, 5.0, 8, 4, a["seed"], flags=abi.MDG_WIDOM_SKIP_OVERLAP, pave=p, inave=n)
    assert c2["inave"].sum() > a["inave"].sum() and np.all(c2["pave"] >= a["pave"])
    c.close()
