"""Energy spectrum and turbulence statistics on the device (ns_spectrum)
against the oracle's restatement of MATLAB_post_processing/PowerSpec.m,
SpecProp.m and KolmoScale.m, through the C ABI.

Tolerances: shell counts exact; spectrum and statistics to a relative 1e-12
(sums of squares in a different order than numpy's)."""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import project, random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,lx", [(32, 2 * np.pi), (64, 2 * np.pi), (32, 3.0)])
def test_spectrum_matches_the_matlab_restatement(n, lx):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    cfg = O.Config(n, n, n, lx=lx, ly=lx, lz=lx, nu=0.01, dt=0.01)
    st = project(random_state(cfg, 81), cfg)
    with Session(make_config(n, n, n, lx=lx, ly=lx, lz=lx, nu=0.01, dt=0.01, scheme=2)) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        k, E, cnt, props = s.spectrum()
        s.step(1)   # the scratch fields it used are free again
        assert np.isfinite(s.get_state(history=False)["u"]).all()
    up, vp, wp = O.cell_centred(st.u, st.v, st.w)
    kr, Er, cr, dk, m = O.power_spec(up, vp, wp, lx)
    pr = O.spec_prop(Er, kr, 0.01, up, vp, wp, n, dk, m)
    assert np.array_equal(cnt, cr)
    assert np.allclose(k, kr, rtol=1e-15, atol=0)
    assert np.max(np.abs(E - Er)) <= 1e-12 * np.max(np.abs(Er))
    for key, val in pr.items():
        assert abs(props[key] - val) <= 1e-12 * abs(val), (key, props[key], val)


def test_spectrum_rejects_non_cubic_boxes():
    from ns_3d_staggered_dp_gb300 import NSError, Session, make_config
    with Session(make_config(32, 16, 32, nu=0.01, dt=0.01, scheme=2)) as s:
        with pytest.raises(NSError) as e:
            s.spectrum()
        assert e.value.status == 1
