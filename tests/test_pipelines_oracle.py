"""The CPU restatement of the MATLAB wrappers (oracle/pipelines.py): the crop
box of cropIndices.m with the wrappers' margins and clamping, and the
composed pipelines' shape and zero-outside-the-box contract."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def pip(port):
    import pipelines
    return pipelines


def test_crop_box_margins_and_clamping(pip):
    m = np.zeros((20, 18, 16), np.uint8, order="F")
    m[5:9, 1:4, 10:16] = 1
    assert pip.crop_box(m, 2) == (slice(3, 11), slice(0, 6), slice(8, 16))
    assert pip.crop_box(m, 1) == (slice(4, 10), slice(0, 5), slice(9, 16))
    with pytest.raises(ValueError):
        pip.crop_box(np.zeros((4, 4, 4), np.uint8), 1)


def test_pipelines_zero_outside_box(pip):
    from qsm_gb300 import synthetic
    rng = np.random.default_rng(0)
    shape = (22, 20, 18)
    m = synthetic.ellipsoid_mask(shape, (5, 6, 4), centre=(9.0, 10.0, 8.0))
    phas = np.asfortranarray(rng.standard_normal(shape + (2,)) * 0.1)
    x = pip.sstgv(phas, m, [1, 1, 1], 1e-3, 2.0, 0.0, 20)
    b = pip.crop_box(m, 2)
    outside = np.ones(shape, bool)
    outside[b] = False
    assert x.shape == phas.shape and not np.any(x[outside]) and np.any(x[b])
    fl = pip.lbv(phas[..., 0], m, [1, 1, 1], maxit=5)
    up, d2 = pip.unwrap_laplacian(phas[..., 0], m, [1, 1, 1])
    b1 = pip.crop_box(m, 1)
    outside1 = np.ones(shape, bool)
    outside1[b1] = False
    for a in (fl, up, d2):
        assert a.shape == shape and not np.any(a[outside1])
