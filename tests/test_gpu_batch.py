"""Batched sweep engine vs the CPU oracle, through the C ABI (GPU only)."""
import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu


def setup_batch(sizes, rng):
    from wavefunctionsimpython_gb300._lib import Batch

    L = 40.0
    b = Batch(sizes, [L] * len(sizes))
    refs = []
    for i, n in enumerate(sizes):
        dx = orc.delta_x((L,) * 3, (n,) * 3)
        U, w = rng.uniform(0.2, 2.0), rng.uniform(1.0, 4.0)
        k0, sig, x0 = rng.uniform(0.5, 3.0), rng.uniform(1.0, 3.0), rng.uniform(-12.0, -6.0)
        b.add_wall(i, U, (0, 0, 0), (1, 0, 0), w)
        b.init_gaussian(i, (sig,) * 3, (x0, 0, 0), (k0, 0, 0))
        V = orc.add_potential_wall(np.zeros((n,) * 3, np.complex64), dx, orc.Wall(potential_hartree=U, plateau_thickness_bohr_radii=w))
        psi0 = orc.gaussian_wave_packet((n,) * 3, dx, (sig,) * 3, (x0, 0, 0), (k0, 0, 0), False)
        refs.append((dx, V, psi0))
    return b, refs


def rel(a, b):
    return float(np.linalg.norm(a.astype(np.complex128) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("swap", [0, 1])
@pytest.mark.parametrize("cluster", [0, 8])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_oracle(graph, cluster, swap):
    """Both step schedules (two passes per size class, cluster setting 0; one cluster
    launch per step) in both radix orientations."""
    rng = np.random.default_rng(11)
    sizes = [32, 48, 32, 64, 96, 48, 128, 32]
    b, refs = setup_batch(sizes, rng)
    b.set_config(cluster, swap)
    b.run(6, 0.01, 1.0, graph=graph)
    b.run(4, 0.01, 1.0, graph=graph)
    for i, (dx, V, psi0) in enumerate(refs):
        ref = orc.split_step(psi0.astype(np.complex128), V, dx, 0.01, 1.0, nsteps=10, double_precision=True)
        assert rel(b.get_psi(i), ref) < 1e-5, f"instance {i} (L={sizes[i]})"


def test_batch_autotune_and_observe():
    rng = np.random.default_rng(5)
    sizes = [32, 64, 48, 96]
    b, refs = setup_batch(sizes, rng)
    psi_before = [b.get_psi(i) for i in range(len(sizes))]
    cl, sw, table = b.autotune(0.01, 1.0, steps=2)
    assert cl in (0, 1, 2, 4, 8, 16) and sw in (0, 1)
    assert table[(cl, sw)] > 0 and table[(cl, sw)] == min(v for v in table.values() if v > 0)
    for i in range(len(sizes)):
        assert np.array_equal(b.get_psi(i), psi_before[i])
    b.run(5, 0.01, 1.0)
    boxes = []
    for n in sizes:
        boxes.append(((n // 2, 0, 0), (n // 2 - 1 if (n // 2) % 2 == 0 else n // 2, n - 1, n - 1)))
    probs = b.observe(boxes)
    for i, (dx, V, psi0) in enumerate(refs):
        psi = orc.split_step(psi0.astype(np.complex128), V, dx, 0.01, 1.0, nsteps=5, double_precision=True)
        assert abs(probs[i] - orc.volume_probability(psi, dx, *boxes[i])) < 1e-6


def test_batch_rejects_unsupported_size():
    from wavefunctionsimpython_gb300._lib import WFS_ERR_UNSUPPORTED, Batch, WfsError

    with pytest.raises(WfsError) as ei:
        Batch([32, 40], [10.0, 10.0])
    assert ei.value.code == WFS_ERR_UNSUPPORTED


@pytest.mark.parametrize("swap", [0, 1])
def test_two_pass_mode_bit_identical_to_cluster_mode(swap):
    """The plane pass of the two-pass mode keeps each yz-plane in shared memory but runs
    the same transforms in the same order as the cluster mode's stages through L2, so
    psi is bit-identical after a run."""
    sizes = [96, 32, 64, 48, 128]
    outs = []
    for cluster in (0, 8):
        b, _ = setup_batch(sizes, np.random.default_rng(3))
        b.set_config(cluster, swap)
        b.run(7, 0.01, 1.0, graph=True)
        outs.append([b.get_psi(i) for i in range(len(sizes))])
    for a, c in zip(*outs):
        assert np.array_equal(a.view(np.uint64), c.view(np.uint64))
