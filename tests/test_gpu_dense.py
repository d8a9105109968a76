"""GPU checks of the dense-vector and 0-d Scalar operations, and of the
B-less reduction reduce(+, A; dims)."""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import csr_from_dense
from helpers import to_dev, to_host, upload

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "finch_kats.json").read_text())["kats"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [0, 1, 1000, 3_000_001])
def test_dot_deterministic(gpu_lib, dtype, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n).astype(dtype)
    y = rng.standard_normal(n).astype(dtype)
    a = to_host(dev.dot(to_dev(x), to_dev(y)))
    b = to_host(dev.dot(to_dev(x), to_dev(y)))
    assert a == b  # same inputs, same bits
    want = float(np.dot(x.astype(np.float64), y.astype(np.float64)))
    scale = float(np.abs(x.astype(np.float64)) @ np.abs(y.astype(np.float64)))
    tol = (1e-13 if dtype == np.float64 else 1e-5) * scale + 1e-30
    assert abs(float(a) - want) <= tol


def test_axpby_map_scalar(gpu_lib):
    rng = np.random.default_rng(0)
    x = rng.standard_normal(5000)
    y = rng.standard_normal(5000)
    a = torch.tensor(0.75, dtype=torch.float64, device="cuda")
    b = torch.tensor(-2.0, dtype=torch.float64, device="cuda")
    out = to_host(dev.axpby(a, to_dev(x), b, to_dev(y)))
    np.testing.assert_allclose(out, 0.75 * x - 2.0 * y, rtol=1e-15, atol=1e-15)
    out = to_host(dev.axpby(a, to_dev(x), None, to_dev(y), signs=1))
    np.testing.assert_allclose(out, -0.75 * x + y, rtol=1e-15, atol=1e-15)
    xi = rng.integers(-100, 100, 777).astype(np.int32)
    yi = rng.integers(-100, 100, 777).astype(np.int32)
    assert np.array_equal(to_host(dev.dense_map(L.MAP_MIN, to_dev(xi), to_dev(yi))), np.minimum(xi, yi))
    assert np.array_equal(to_host(dev.dense_map(L.MAP_SUB, to_dev(xi), to_dev(yi))), xi - yi)
    q = to_host(dev.scalar_op(L.MAP_DIV, a, b))
    assert float(q) == 0.75 / -2.0


@pytest.mark.parametrize("dims,key", [(1, "dims1"), (2, "dims2"), (0, "all")])
def test_reduce_kat_without_b(gpu_lib, dims, key):
    k = KATS["reduce"]
    A = upload(csr_from_dense(np.array(k["A"])))
    want = k[key] if isinstance(k[key], list) else [k[key]]
    np.testing.assert_allclose(to_host(dev.ewise_reduce(dims, A)), want, rtol=1e-15)
