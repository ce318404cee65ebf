"""The C++/OpenMP restatement of the reference step (oracle/ns_ref_cpu.cpp,
the timed CPU baseline) against the NumPy oracle: two independent
restatements of big_periodic_3D.f90:326-567 agree to rounding."""
import numpy as np
import pytest

from oracle import ns_oracle as O
from oracle.ns_ref_cpu import CpuStep
from tests.helpers import project, random_state, rel_l2


@pytest.mark.parametrize("scheme", [O.AB2_CN, O.AB2, O.EULER])
@pytest.mark.parametrize("dpf", [0, 1])
def test_cpp_step_matches_numpy_oracle(scheme, dpf):
    cfg = O.Config(16, 8, 32, lx=2 * np.pi, ly=1.3, lz=3.0, nu=0.03, dt=0.01, scheme=scheme, dp_flag=dpf)
    st = project(random_state(cfg, 101), cfg)
    ref = st.copy()
    cpu = CpuStep(cfg)
    for _ in range(4):
        ref = O.step(ref, cfg)
        cpu.step(st)
    for name in ("u", "v", "w", "p", "px", "py", "pz"):
        assert rel_l2(getattr(st, name), getattr(ref, name)) < 1e-12, name
