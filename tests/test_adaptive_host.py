"""Host side of the adaptive leaf-flux drop-in (no GPU): the context manager
swaps the adaptive module's ``rusanov`` for the GPU batch function and puts
the original back, also when the block raises."""

import types

import pytest

from torch_gb300 import adaptive


def test_gpu_leaf_fluxes_swaps_and_restores_the_module_flux():
    def cpu_flux(left, right, gl, gr, direction):
        return "cpu"

    module = types.SimpleNamespace(rusanov=cpu_flux)
    with adaptive.gpu_leaf_fluxes(module):
        assert module.rusanov is not cpu_flux
    assert module.rusanov is cpu_flux
    with pytest.raises(RuntimeError):
        with adaptive.gpu_leaf_fluxes(module, precision="fp32"):
            raise RuntimeError("step failed")
    assert module.rusanov is cpu_flux


def test_leaf_fluxes_rejects_bad_batches_before_touching_the_gpu():
    import numpy as np

    with pytest.raises(ValueError):
        adaptive.leaf_fluxes(np.ones((4, 3)), np.ones((4, 2)), 1.4, 1.4, 0)
    with pytest.raises(ValueError):
        adaptive.leaf_fluxes(np.ones((4, 3)), np.ones((4, 3)), 1.4, 1.4, 2)
