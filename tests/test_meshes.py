"""Workload generators: element counts and block-pattern sizes of the measured configurations."""
import numpy as np

from bounce_softbody_gb300 import meshes


def nnzb(desc):
    pairs = set()
    for e in desc.tets:
        for a in e:
            for b in e:
                pairs.add((int(a), int(b)))
    for e in desc.tris:
        for a in e:
            for b in e:
                pairs.add((int(a), int(b)))
    for a, b in desc.springs:
        pairs.update({(int(a), int(b)), (int(b), int(a)), (int(a), int(a)), (int(b), int(b))})
    return len(pairs)


def test_tet10_counts():
    d = meshes.config_tet10()
    assert d.n == 1000 and d.tets.shape == (4374, 4)
    assert (d.type == meshes.STATIC).sum() == 100
    assert nnzb(d) == 12718


def test_kuhn_orientation_and_jitter():
    d = meshes.tet_grid(5, 4, 3, spacing=0.1, jitter=0.01, seed=1)
    e = d.x[d.tets[:, 1:].astype(int)] - d.x[d.tets[:, :1].astype(int)]
    vol = np.linalg.det(e) / 6.0
    assert (vol > 0).all()
    grid = d.x / 0.1
    assert np.abs(grid - np.round(grid)).max() <= 0.0100001


def test_cloth128_counts():
    d = meshes.config_cloth128()
    assert d.n == 16384 and d.tris.shape[0] == 32258 and d.springs.shape[0] == 64768
    assert (d.type == meshes.STATIC).sum() == 2


def test_tet64_nnzb_formula():
    # nnzb = n + 2 E for a Kuhn grid: axis + face-diagonal + body-diagonal edges
    a = 64
    E = 3 * a * a * (a - 1) + 3 * a * (a - 1) ** 2 + (a - 1) ** 3
    assert a ** 3 + 2 * E == 3834622
    assert meshes.kuhn_cells(a, a, a).shape[0] == 1500282


def test_batch_sizes_are_seeded():
    a = meshes.batch_bodies(8, seed=3)
    b = meshes.batch_bodies(8, seed=3)
    assert [x.n for x in a] == [x.n for x in b]
    assert all(4 ** 3 <= x.n <= 40 ** 3 for x in a)
    np.testing.assert_array_equal(a[3].x, b[3].x)
