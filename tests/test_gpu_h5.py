"""Session snapshots in the reference's HDF5 layout (ns_h5_write_state,
big_periodic_3D.f90:630-651) and restarts from them (ns_h5_read_state,
:296-324), through the C ABI on the GPU."""
import numpy as np
import pytest

from oracle import ns_h5 as H
from oracle import ns_oracle as O
from tests.helpers import random_state

pytestmark = pytest.mark.gpu


def session(cfg):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    return Session(make_config(cfg.nx, cfg.ny, cfg.nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, nu=cfg.nu, dt=cfg.dt,
                               scheme=cfg.scheme, bc=cfg.bc, pbc=cfg.pbc, dp_flag=cfg.dp_flag))


def test_snapshot_has_the_reference_layout(tmp_path):
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2_CN)
    st = random_state(cfg, 7, history=True)
    p = tmp_path / "snap.h5"
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
        s.step(2)
        ref = s.get_state()
        s.h5_write_state(p, time=0.02, time_step=2)
    g = H.read(str(p))
    assert list(g.attrs) == ["nx", "dt", "nu", "time_scheme", "time_step", "time"]
    assert g.attrs["nx"][0] == 16 and g.attrs["dt"][0] == 0.01 and g.attrs["nu"][0] == 0.02
    assert g.attrs["time_scheme"] == "AB2-CN" and g.attrs["time_step"][0] == 2 and g.attrs["time"][0] == 0.02
    names = {"u": "u", "v": "v", "w": "w", "p": "p", "hx": "rhs_x_previous", "hy": "rhs_y_previous",
             "hz": "rhs_z_previous"}
    for k, n in names.items():
        d = g.members[n]
        assert d.shape == ref[k].shape[::-1]
        assert d.data.tobytes() == np.asfortranarray(ref[k]).tobytes(order="F")


@pytest.mark.parametrize("scheme", [O.AB2, O.AB2_CN])
def test_restart_continues_bit_for_bit(tmp_path, scheme):
    """Three steps in one run give the bits of one step, a snapshot, a
    restart in a new session and two more steps (the history carries the
    AB2 part across)."""
    cfg = O.Config(32, 16, 16, nu=0.02, dt=0.01, scheme=scheme, bc=(1, 2, 1), pbc=(1, 3, 1))
    st = random_state(cfg, 13, history=True)
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
        s.step(3)
        ref = s.get_state()
    p = tmp_path / "restart.h5"
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
        s.step(1)
        s.h5_write_state(p, time=0.01, time_step=1)
    with session(cfg) as s:
        t, ts = s.h5_read_state(p)
        assert (t, ts) == (0.01, 1)
        assert s.diag()["euler_start_pending"] == 0
        s.step(2)
        got = s.get_state()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


def test_init_file_without_history_is_an_euler_start(tmp_path):
    """The init file of :296-301 holds u, v, w, p only: the restart's first
    step is the Euler start, as after ns_set_state without history."""
    from ns_3d_staggered_dp_gb300 import H5File
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2_CN)
    st = random_state(cfg, 17)
    p = tmp_path / "init.h5"
    with H5File(p, "w") as f:
        for k in ("u", "v", "w", "p"):
            f.write(k, getattr(st, k))
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(2)
        ref = s.get_state()
    with session(cfg) as s:
        assert s.h5_read_state(p) == (0.0, 0)
        assert s.diag()["euler_start_pending"] == 1
        s.step(2)
        got = s.get_state()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


def test_snapshot_of_another_grid_is_refused(tmp_path):
    from ns_3d_staggered_dp_gb300 import NSError
    p = tmp_path / "s16.h5"
    c16 = O.Config(16, 16, 16, nu=0.02, dt=0.01)
    with session(c16) as s:
        st = random_state(c16, 1)
        s.set_state(st.u, st.v, st.w, st.p)
        s.h5_write_state(p)
        with pytest.raises(NSError) as e:
            s.h5_write_state(p)  # exists
        assert e.value.status == 8
        s.h5_write_state(p, overwrite=True)
    with session(O.Config(32, 16, 16, nu=0.02, dt=0.01)) as s:
        with pytest.raises(NSError) as e:
            s.h5_read_state(p)
        assert e.value.status == 1
