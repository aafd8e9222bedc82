"""The `cupano` names on the GPU: compute_laplacian against the oracle's Laplacian and the reference
tests' known answer, and the reference's own Python stitcher tests run against this library.

The reference's test file (tests/python/test_pytorch_pano.py of hm-cupano) is not part of this
repository: the suite test runs it where the environment variable HMP_CUPANO_TESTS names a
directory holding that file, with this library's `cupano` package first on the import path, and is
skipped otherwise. Its sibling test_triton_backend.py is not run: it imports the reference's
internal torch and Triton operators (cupano.ops._remap_to_canvas_torch, cupano.triton_ops), which
are not part of the stitcher API this library replaces.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def test_compute_laplacian_matches_the_oracle(oracle_lib):
    import torch
    from cupano.ops import compute_laplacian

    rng = np.random.default_rng(9)
    for hw, hh in ((37, 23), (64, 64), (5, 9)):
        lw, lh = (hw + 1) // 2, (hh + 1) // 2
        high = rng.uniform(0, 255, (hh, hw, 4)).astype(np.float32)
        low = rng.uniform(0, 255, (lh, lw, 4)).astype(np.float32)
        high[rng.random((hh, hw)) < 0.2, 3] = 0
        low[rng.random((lh, lw)) < 0.3, 3] = 0
        want = oracle_lib.laplacian_rgba(high, low)
        for dev in ("cpu", "cuda"):
            got = compute_laplacian(torch.from_numpy(high)[None].to(dev), torch.from_numpy(low)[None].to(dev))
            assert got.device.type == dev
            assert np.array_equal(got[0].cpu().numpy(), want), (hw, hh, dev)


def test_compute_laplacian_renormalises_alpha_weights():
    """The known answer of the reference's test (test_pytorch_pano.py:192-201): a single opaque
    low pixel under a transparent high level."""
    import torch
    from cupano.ops import compute_laplacian

    high = torch.zeros((1, 4, 4, 4))
    low = torch.zeros((1, 2, 2, 4))
    low[:, 1, 1, :] = torch.tensor([100.0, 110.0, 120.0, 255.0])
    lap = compute_laplacian(high, low, backend="auto")
    assert torch.equal(lap[0, 1, 1, :3], torch.tensor([-100.0, -110.0, -120.0]))
    assert lap[0, 1, 1, 3].item() == 0.0


def test_reference_python_suite_against_this_library():
    d = os.environ.get("HMP_CUPANO_TESTS")
    suite = Path(d) / "test_pytorch_pano.py" if d else None
    if suite is None or not suite.exists():
        pytest.skip("HMP_CUPANO_TESTS does not name a directory holding the reference's test_pytorch_pano.py")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(REPO / "hm-cupano_gb300"), env_path()]))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-rA", str(suite)],
                       capture_output=True, text=True, env=env, cwd=str(suite.parent), timeout=900)
    out = r.stdout + r.stderr
    print(out[-4000:])
    m = re.search(r"(\d+) passed", out)
    assert r.returncode == 0 and m and int(m.group(1)) >= 6 and "failed" not in out, out[-3000:]


def env_path() -> str:
    return os.environ.get("PYTHONPATH", "")
