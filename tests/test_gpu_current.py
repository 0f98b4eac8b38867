"""Plane probability current on the GPU vs the CPU oracle (GPU only)."""
import math

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("normal,center", [((1, 0, 0), (0.0, 0.0, 0.0)), ((1, 1, 0), (0.5, -1.0, 0.3)),
                                           ((0, 1, 0), (0.0, 2.0, 0.0))])
def test_plane_current_matches_oracle(normal, center, dbl):
    from wavefunctionsimpython_gb300 import Engine

    n, L = (48, 32, 64), (24.0, 16.0, 32.0)
    dx = orc.delta_x(L, n)
    e = Engine(n, L, double_precision=dbl)
    e.init_gaussian((2.0, 1.8, 2.2), (-1.0, 0.5, 0.0), (1.5, 0.7, 0.0))
    e.add_wall(2.0, (2.0, 0, 0), (1, 0, 0), 1.0)
    e.step_split(4, 0.02, 1.0)
    psi = e.get_psi()
    size, count = (14.0, 12.0), (63, 51)
    got = e.plane_current(center, normal, size, count, 1.0)
    ref, _ = orc.plane_probability_current(psi, dx, center, normal, size, count, 1.0)
    assert abs(got - ref) <= 2e-5 * max(1.0, abs(ref))


def test_plane_current_free_packet_flux():
    """A packet moving along x crosses a plane through its centre with flux ~ k/m * (2 pi sigma^2)^(-1/2)."""
    from wavefunctionsimpython_gb300 import Engine

    n, L = (64, 64, 64), (32.0, 32.0, 32.0)
    e = Engine(n, L, double_precision=True)
    e.init_gaussian((2.0,) * 3, (0.0, 0.0, 0.0), (1.5, 0.0, 0.0))
    got = e.plane_current((0, 0, 0), (1, 0, 0), (24.0, 24.0), (97, 97), 1.0)
    assert abs(got - 1.5 / (math.sqrt(2 * math.pi) * 2.0)) < 2e-3


@pytest.mark.parametrize("dbl", [False, True])
def test_device_loop_records_plane_currents(dbl):
    """run_split_planes: fluxes through two planes, a volume probability and the expected
    location recorded on the device every third step, against the oracle along the same
    trajectory."""
    from wavefunctionsimpython_gb300 import Engine

    n, L = (48, 32, 64), (24.0, 16.0, 32.0)
    dx = orc.delta_x(L, n)
    e = Engine(n, L, double_precision=dbl)
    e.init_gaussian((2.0, 1.8, 2.2), (-1.0, 0.5, 0.0), (1.5, 0.7, 0.0))
    e.add_wall(2.0, (2.0, 0, 0), (1, 0, 0), 1.0)
    V = e.get_potential()
    psi = e.get_psi().astype(np.complex128)
    planes = [((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (14.0, 12.0), (63, 51)),
              ((0.5, -1.0, 0.3), (1.0, 1.0, 0.0), (10.0, 10.0), (41, 41))]
    box, loc = ((2, 2, 2), (43, 27, 59)), ((1, 1, 1), (45, 29, 61))
    ps, ls, fs = e.run_split_planes(12, 0.02, 1.0, 3, [box], loc, planes)
    assert fs.shape == (4, 2)
    tol = 1e-9 if dbl else 2e-5
    for k in range(4):
        for p, (c, nrm, size, count) in enumerate(planes):
            ref, _ = orc.plane_probability_current(psi.astype(np.complex128 if dbl else np.complex64), dx, c, nrm,
                                                   size, count, 1.0)
            assert abs(fs[k, p] - ref) <= tol * max(1.0, abs(ref)), (k, p, fs[k, p], ref)
        assert abs(ps[k, 0] - orc.volume_probability(psi, dx, *box)) < (1e-10 if dbl else 1e-6)
        psi = orc.split_step(psi, V, dx, 0.02, 1.0, nsteps=3)
    assert np.linalg.norm(e.get_psi() - psi) / np.linalg.norm(psi) < (1e-11 if dbl else 1e-5)
    e.close()
