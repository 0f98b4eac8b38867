"""Copy-staged strided pass against the cp.async pipelined pass (GPU only).

The two kernels run the same butterflies in the same order. They differ only in
how each tile reaches shared memory: one tensor copy issued by one thread, or
one cp.async per element. So a split-step run must give bit-identical psi on
both paths. The path is chosen once per process (WFS_STRIDED_STAGED=0 selects
cp.async), so each side runs in a child process through the C ABI.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from wavefunctionsimpython_gb300 import Engine

n = tuple(int(v) for v in sys.argv[2].split(","))
L = tuple(0.4 * v for v in n)
rng = np.random.default_rng(7)
V = (rng.uniform(0.0, 2.0, n) - 0.3j * rng.uniform(0.0, 1.0, n)).astype(np.complex64)
e = Engine(n, L)
e.set_potential(V)
e.init_gaussian((0.12 * L[0], 0.11 * L[1], 0.1 * L[2]), (-0.1 * L[0], 0.05 * L[1], 0.0), (2.0, 0.5, -0.5))
e.step_split(5, 0.01, 1.0)
np.save(sys.argv[3], e.get_psi())
"""


def _run(n, staged, path):
    env = dict(os.environ, WFS_STRIDED_STAGED="1" if staged else "0")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, ",".join(map(str, n)), str(path)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


# (64, 128, 128): x pass over 512 tiles with the fused plane pass; (256, 96, 96): 576 x tiles
# of 16 columns; (384, 64, 6): per-axis schedule, y tiles of 32 columns with 6 in the grid
@pytest.mark.parametrize("n", [(64, 128, 128), (256, 96, 96), (384, 64, 6)])
def test_staged_pass_bit_identical_to_cp_async(n, tmp_path):
    a = _run(n, True, tmp_path / "staged.npy")
    b = _run(n, False, tmp_path / "cp_async.npy")
    assert a.dtype == np.complex64 and a.shape == n
    assert np.isfinite(a).all()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_expired_tile_wait_reports_timeout_once_and_recovers():
    """The expiry path of the copy-staged pass, made to run without any fault: a wait
    limit of zero makes every tile wait give up at once. The pass must return (each CTA
    stops after its first tile and drains its two copies in flight), the next
    synchronisation must report WFS_ERR_TIMEOUT exactly once, and with the default limit
    restored the engine must step correctly again."""
    import time

    from oracle import wfs_oracle as orc
    from wavefunctionsimpython_gb300 import Engine
    from wavefunctionsimpython_gb300._lib import WfsError

    n, L = (64, 128, 128), (25.6, 51.2, 51.2)
    e = Engine(n, L)
    e.init_gaussian((3.0, 5.0, 5.0), (-3.0, 2.0, 0.0), (1.5, 0.5, 0.0))
    psi0 = e.get_psi()
    e.set_copy_wait_limit(0.0)
    t0 = time.perf_counter()
    e.step_split(1, 0.01, 1.0)
    with pytest.raises(WfsError) as exc:
        e.synchronize()
    assert exc.value.code == 3  # WFS_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    e.synchronize()  # reported once: the status word was cleared
    e.set_copy_wait_limit(1.0)
    e.set_psi(psi0)
    e.step_split(3, 0.01, 1.0)
    e.synchronize()
    dx = orc.delta_x(L, n)
    ref = orc.split_step(psi0.astype(np.complex128), np.zeros(n, np.complex64), dx, 0.01, 1.0, nsteps=3)
    got = e.get_psi()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    e.close()
