"""Oracle restatement of the animator's frame (CPU): draw order, colour ramp,
disk coverage."""
import numpy as np

from oracle import oracle as O


def test_quicksort_draw_order_is_descending_z():
    rng = np.random.default_rng(4)
    for n in (1, 2, 3, 17, 1000):
        z = rng.choice(2**62, size=n, replace=False).astype(np.int64)
        order = O.draw_order(z)
        assert np.array_equal(order, np.argsort(-z, kind="stable"))


def test_quicksort_with_equal_keys_is_a_permutation_sorted_by_key():
    z = np.array([5, 1, 5, 3, 3, 9, 1, 1], np.int64)
    order = O.draw_order(z)
    assert sorted(order.tolist()) == list(range(len(z)))
    assert np.all(np.diff(-z[order]) >= 0)


def para_ramp(i):
    """gx/graphics.go:156-164 restated in Python floats (no contraction)."""
    x = float(i)
    r = min(215.0, max(0.0, -abs((x - 60) * 31 / 17 - 232) + 245))
    g = min(190.0, max(0.0, -abs(x * 31 / 17 - 232) + 245))
    b = min(215.0, max(0.0, -abs((x + 70) * 31 / 17 - 232) + 245))
    return int(r), int(g), int(b)


def test_single_disk_pixels_and_colour():
    # one particle at pixel centre (100, 50) of a 200 x 100 canvas: radius-4 disk
    x, y = np.array([0.5]), np.array([0.5])
    mass = 1.0
    rho = np.array([0.05])  # rho / (m N 10) * 256 = 1.28 -> index 1
    img = O.render(x, y, rho, mass, np.array([0]), 200, 100)
    covered = np.argwhere(img[:, :, 0:3].any(axis=2) | (img[:, :, 3] == 255) & (img.sum(axis=2) != 255))
    yy, xx = np.mgrid[0:100, 0:200]
    disk = ((xx - 100.0) ** 2 + (yy - 50.0) ** 2) <= 16
    col = np.array(para_ramp(1) + (255,), np.uint8)
    assert np.all(img[disk] == col)
    assert np.all(img[~disk] == np.array([0, 0, 0, 255], np.uint8))
    assert disk.sum() == 49
    del covered


def test_later_disks_paint_over_earlier_ones_and_clip():
    x = np.array([0.0, 0.01, 0.999])
    y = np.array([0.0, 0.0, 0.5])
    rho = np.array([0.0, 100.0, 3.0])
    img_a = O.render(x, y, rho, 1.0, np.array([0, 1, 2]), 100, 50)
    img_b = O.render(x, y, rho, 1.0, np.array([1, 0, 2]), 100, 50)
    assert not np.array_equal(img_a, img_b)  # the overlap shows the later disk
    assert tuple(img_a[0, 1, :3]) == para_ramp(255)  # particle 1 (clamped index) on top
    assert tuple(img_b[0, 0, :3]) == para_ramp(0)
    assert img_a.shape == (50, 100, 4) and np.all(img_a[:, :, 3] == 255)
