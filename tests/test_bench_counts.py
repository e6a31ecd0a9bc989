"""The MG-PCG roofline's operation count (bench.py:mgpcg_fp64_ops) on the CPU:
its numpy restatements of the next-level mask and of the boundary band equal
the oracle's coarsen_grid_mex and boundary_mask_mex on random, ellipsoidal and
full masks of odd and even sizes, and the count of the benchmark's problem is
stable."""
import sys

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as b
    return b


def _masks(rng, shape):
    import qsm_gb300.synthetic as S

    full = np.zeros(shape, bool)
    full[1:-1, 1:-1, 1:-1] = True
    _, ell, _ = S.poisson_case(shape, 3, semi=(3.0, 20.0))
    return {"random": rng.random(shape) < 0.8, "ellipsoid": ell != 0, "full": full}


@pytest.mark.parametrize("shape", [(20, 17, 13), (31, 30, 29), (16, 16, 16), (9, 12, 7), (8, 8, 9)])
def test_mask_rules_match_oracle(bench, port, shape):
    rng = np.random.default_rng(sum(shape))
    for name, G in _masks(rng, shape).items():
        Gp = np.asfortranarray(G.astype(np.uint8))
        n2 = tuple(((m - 2 + 1) >> 1) + 2 for m in shape)
        ref = np.zeros(n2, np.uint8, order="F")
        port.coarsen_grid_mex(ref, Gp)
        assert np.array_equal(bench._coarsen(G), ref != 0), (shape, name, "coarsen")
        refb = np.zeros(shape, np.uint8, order="F")
        port.boundary_mask_mex(refb, Gp)
        assert np.array_equal(bench._band(G), refb != 0), (shape, name, "band")


def test_benchmark_operation_count(bench):
    import qsm_gb300.synthetic as S

    _, mask, _ = S.config1(seed=1)
    ops = bench.mgpcg_fp64_ops(mask)
    # 12 per padded voxel and 10 per G voxel in the PCG steps, the rest in two V-cycles
    assert 1.0e9 < ops < 1.1e9
    assert bench.mgpcg_fp64_ops(mask, coarse_outer_per_cycle=2) > ops


def test_recorded_traffic_matches_the_kernel_sources(bench):
    """The DRAM traffic bench.py reports for the headline kernel was captured
    from the current kernel sources: its key carries the digest of the
    sources without comments, so an edited kernel needs a new capture (the
    bench would otherwise report traffic null)."""
    digest = bench.kernel_digest()
    keys = [k for k in bench.NCU_TRAFFIC_224x224x128 if k[0] == digest]
    assert keys, f"no ncu traffic recorded for kernel digest {digest}"
    assert all(150e6 < bench.NCU_TRAFFIC_224x224x128[k] < 600e6 for k in keys)
