"""Install the unmodified TORCH reference into baseline/_ref.

`bench.py --impl reference` (and the CPU baseline of the default run) time
the reference's own NumPy step from baseline/_ref when it is there.  The
reference tree has neither setup.py nor pyproject.toml, so

    python -m pip install --no-index --no-build-isolation \
        --find-links /opt/wheelhouse --target baseline/_ref <reference>

refuses it ("Neither 'setup.py' nor 'pyproject.toml' found").  This script
copies the tree to a temporary directory, adds a pyproject.toml that declares
the package directory python/cfdSolver (no reference file is changed), and
runs the same offline install from the copy with --no-deps (the reference's
plotting and HDF5 requirements are not on the step's path and are not in the
wheelhouse).

    python baseline/install_reference.py [--reference PATH]

PATH defaults to $TORCH_REFERENCE, else /root/reference.  The install holds
Python files only, so it runs unchanged on any host architecture.
"""

import argparse
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
PYPROJECT = """[build-system]
requires = ["setuptools"]
build-backend = "setuptools.build_meta"

[project]
name = "torch-reference"
version = "0"

[tool.setuptools]
package-dir = {"" = "python"}
packages = ["cfdSolver"]
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("TORCH_REFERENCE", "/root/reference"))
    ap.add_argument("--target", default=str(HERE / "_ref"))
    args = ap.parse_args()
    src = Path(args.reference)
    if not (src / "python" / "cfdSolver").is_dir():
        sys.exit(f"{src} holds no python/cfdSolver")
    with tempfile.TemporaryDirectory() as tmp:
        copy = Path(tmp) / "reference"
        shutil.copytree(src, copy, ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
        (copy / "pyproject.toml").write_text(PYPROJECT)
        cmd = [sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation",
               "--no-deps", "--find-links", "/opt/wheelhouse", "--target", args.target,
               "--upgrade", str(copy)]
        subprocess.run(cmd, check=True)
    print("installed", Path(args.target) / "cfdSolver")


if __name__ == "__main__":
    main()
