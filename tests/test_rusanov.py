"""Rusanov fluxes (python/cfdSolver/torchFlux.py:80-122): the GPU drop-in
against the reference's own rusanov_flux on seeded random faces and on the
leaf-face batches an adaptive session hands to it (tests/golden/rusanov.npz,
recorded by tests/golden/make_golden.py).  Double precision is bitwise; the
host test checks the oracle restatement against the same vectors."""

from pathlib import Path

import numpy as np
import pytest

from oracle import metric as M

GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "rusanov.npz")
CASES = sorted({k.split("|")[0] for k in G.files})


def direction(key):
    if key.startswith("amr"):
        return int(G[f"{key}|dir"][0])
    return int(key.split("dir")[1])


@pytest.mark.parametrize("key", CASES)
def test_oracle_rusanov_matches_reference(key):
    out = M.rusanov(G[f"{key}|left"], G[f"{key}|right"], G[f"{key}|gl"], G[f"{key}|gr"],
                    direction(key))
    np.testing.assert_array_equal(out, G[f"{key}|flux"])


@pytest.mark.gpu
@pytest.mark.parametrize("key", CASES)
def test_gpu_rusanov_matches_reference_bitwise(key):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import torch_gb300
    args = (G[f"{key}|left"], G[f"{key}|right"], G[f"{key}|gl"], G[f"{key}|gr"], direction(key))
    np.testing.assert_array_equal(torch_gb300.rusanov_flux(*args), G[f"{key}|flux"])
    grid = torch_gb300.rusanov_flux_grid(*args)
    np.testing.assert_array_equal(grid, G[f"{key}|flux"])
    f32 = torch_gb300.rusanov_flux(*args, precision="fp32")
    ref = G[f"{key}|flux"]
    np.testing.assert_allclose(f32, ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_rusanov_rejects_bad_shapes():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import torch_gb300
    a = np.ones((4, 3))
    with pytest.raises(ValueError):
        torch_gb300.rusanov_flux(a, np.ones((4, 2)), 1.4, 1.4, 0)
    with pytest.raises(ValueError):
        torch_gb300.rusanov_flux(a, a, 1.4, 1.4, 2)
