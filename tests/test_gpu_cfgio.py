"""Configuration files and checkpoints of the resident state: the library's .cfg writer read back
by the Python reader of the reference format (config_input), the library's reader against the
Python reader on the same file, and a run continued from a binary checkpoint."""
import os

import numpy as np
import pytest

from md_sim_gb300 import abi, configs
from md_sim_gb300 import system as S

pytestmark = pytest.mark.gpu


def _cases():
    return {"slab": lambda: configs.slab_water(nwat=256, cells=5, placement="lattice", kmax=5),
            "shake": lambda: configs.shake_water(nwat=256, cells=6),
            "electrolyte": lambda: configs.slab_electrolyte(nwat=128, npair=4, cells=4, kmax=4)}


def _same_state(a, b, rtol):
    for name in ("c", "q", "w"):
        x, y = getattr(a, name)[..., : a.nrig], getattr(b, name)[..., : b.nrig]
        if y.size:
            assert np.allclose(x, y, rtol=rtol, atol=rtol * (np.abs(y).max() + 1e-300)), name
    # sites of rigid molecules are rebuilt from the centre and quaternion on reading (config_init);
    # positions of the other moving atoms are written as they are
    for name in ("x0", "y0", "z0"):
        x, y = getattr(a, name)[a.nriga: a.nmove], getattr(b, name)[b.nriga: b.nmove]
        assert np.allclose(x, y, rtol=0, atol=rtol * 100.0), name
    n0, n1 = a.nriga, a.nliqa
    if n1 > n0:
        xa, xb = a.xd[:, :, n0:n1], b.xd[:, :, n0:n1]
        assert np.allclose(xa, xb, rtol=rtol, atol=rtol * (np.abs(xb).max() + 1e-300))
    assert np.allclose(a.s, b.s, rtol=rtol, atol=1e-300) and np.allclose(a.rs, b.rs, rtol=rtol, atol=1e-300)


@pytest.mark.parametrize("name", ["slab", "shake", "electrolyte"])
@pytest.mark.parametrize("full", [True, False])
def test_write_cfg_reads_back(name, full, gpulib, tmp_path):
    s, prm = _cases()[name]()
    ctx = abi.Context(gpulib, s.copy(), prm)
    ctx.set_state(s.copy())
    ctx.run(4)
    ref = ctx.get_state(s.copy())
    path = str(tmp_path / "out.cfg")
    ctx.write_cfg(path, full_precision=full)
    with open(path) as fh:
        back = S.parse_cfg(fh.read(), s.fld, s.top, s.dt)
    _same_state(back, ref, 1e-15 if full else 2e-8)
    ctx.close()


@pytest.mark.parametrize("name", ["slab", "shake", "electrolyte"])
def test_read_cfg_matches_python_reader(name, gpulib, tmp_path):
    s, prm = _cases()[name]()
    path = str(tmp_path / "in.cfg")
    with open(path, "w") as fh:
        fh.write(S.write_cfg(s))
    with open(path) as fh:
        py = S.parse_cfg(fh.read(), s.fld, s.top, s.dt)
    py.shake_init()  # the reference's start-up after config_input (src/move.f90:394-396)
    a = abi.Context(gpulib, s.copy(), prm)
    a.read_cfg(path, s)
    got = a.get_state(s.copy())
    b = abi.Context(gpulib, py.copy(), prm)
    b.set_state(py)
    want = b.get_state(py.copy())
    _same_state(got, want, 1e-14)
    # both step the same (the site offsets rsx are rebuilt by the predictor of the first step)
    ra, rb = a.run(3), b.run(3)
    assert abs(ra["htot"] - rb["htot"]) <= 1e-9 * abs(rb["htot"])
    a.close()
    b.close()


def test_checkpoint_continues_the_run(gpulib, tmp_path):
    s, prm = configs.slab_water(nwat=256, cells=5, placement="lattice", kmax=5)
    a = abi.Context(gpulib, s.copy(), prm)
    a.set_state(s.copy())
    a.run(8)
    path = str(tmp_path / "state.ckpt")
    a.checkpoint_save(path)
    ra = a.run(12)
    sa = a.get_state(s.copy())
    b = abi.Context(gpulib, s.copy(), prm)
    b.checkpoint_load(path)
    rb = b.run(12)
    sb = b.get_state(s.copy())
    assert rb["steps"] == ra["steps"] == 20
    assert abs(ra["htot"] - rb["htot"]) <= 1e-9 * abs(ra["htot"])
    assert np.abs(sa.x0[: s.nmove] - sb.x0[: s.nmove]).max() < 1e-8
    with pytest.raises(abi.MdgError):
        other = configs.slab_water(nwat=128, cells=5, placement="lattice", kmax=5)
        abi.Context(gpulib, other[0], other[1]).checkpoint_load(path)
    a.close()
    b.close()
