"""The oracle's rectangularize restatement pinned against the reference's own test
(unwrap/src/metrics.rs:258-279).  CPU only."""
import numpy as np

from oracle import oracle as O


def test_rectangularize_open_square_fits_the_unit_square():
    uv = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    q, ext = O.rectangularize(uv, [1, 1, 1, 1])
    assert abs(ext[0] - 1.0) < 1e-9 and abs(ext[1] - 1.0) < 1e-9
    for u, v in q:
        assert min(abs(u), abs(1 - u), abs(v), abs(1 - v)) < 1e-9


def test_rectangularize_rotated_rectangle_is_straightened():
    """A 2 x 1 rectangle rotated by 30 degrees: the ladder finds the axis-aligned fit, every
    interior point stays inside [0,1]^2 and every border point lands on a side."""
    t = np.deg2rad(30.0)
    R = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    g = np.array([[x, y] for y in np.linspace(0, 1, 6) for x in np.linspace(0, 2, 11)])
    border = ((g[:, 0] == 0) | (g[:, 0] == 2) | (g[:, 1] == 0) | (g[:, 1] == 1)).astype(int)
    q, ext = O.rectangularize(g @ R.T, border)
    assert np.all(q >= -1e-12) and np.all(q <= 1 + 1e-12)
    on_side = np.minimum.reduce([np.abs(q[:, 0]), np.abs(1 - q[:, 0]), np.abs(q[:, 1]), np.abs(1 - q[:, 1])])
    assert np.all(on_side[border == 1] == 0.0)
    assert sorted(np.round(ext, 1)) == [1.0, 2.0]


def test_rectangularize_without_border_normalises_the_box():
    uv = np.array([[2.0, 1.0], [4.0, 1.0], [3.0, 5.0]])
    q, ext = O.rectangularize(uv, [0, 0, 0])
    assert np.allclose(ext, [2.0, 4.0]) and np.allclose(q, [[0, 0], [1, 0], [0.5, 1]])
