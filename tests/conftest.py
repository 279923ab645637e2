import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


import types  # noqa: E402

import numpy as np  # noqa: E402
import pytest  # noqa: E402


class _NpzHDF5(types.ModuleType):
    """An h5py stand-in for checkpoint tests (h5py is not installed): the
    datasets of a "file" are NumPy arrays kept in an .npz container, with the
    subset of h5py's File interface the checkpoint reader and writer use
    (modes r / w / r+, item get / set / delete, groups listed by name)."""

    class File:
        def __init__(self, path, mode="r"):
            self.path, self.mode, self.data = str(path), mode, {}
            if mode in ("r", "r+"):
                with np.load(self.path) as z:
                    self.data = {k.replace("|", "/"): z[k] for k in z.files}

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            if self.mode in ("w", "r+") and exc[0] is None:
                with open(self.path, "wb") as f:
                    np.savez(f, **{k.replace("/", "|"): v for k, v in self.data.items()})

        def create_dataset(self, name, data, **options):
            self.data[name] = np.array(data)

        def flush(self):
            pass

        def __setitem__(self, name, value):
            self.data[name] = np.array(value)

        def __delitem__(self, name):
            del self.data[name]

        def __getitem__(self, name):
            if name in self.data:
                return self.data[name]
            members = [k[len(name) + 1:] for k in self.data if k.startswith(name + "/")]
            if not members:
                raise KeyError(name)
            return members


@pytest.fixture
def fake_h5py(monkeypatch):
    module = _NpzHDF5("h5py")
    monkeypatch.setitem(sys.modules, "h5py", module)
    return module
