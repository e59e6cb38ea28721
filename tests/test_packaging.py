"""Packaging: a wheel built from the repository carries the Python package
and the compiled library (setup.py runs icm_gb300/build.py first).  Built
from a copy of the sources with their compiled objects, so nothing is
recompiled and the repository stays clean."""
import os
import shutil
import subprocess
import sys
import zipfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_wheel_carries_library(tmp_path):
    pytest.importorskip("setuptools")
    pytest.importorskip("wheel")
    from icm_gb300 import build as b
    b.build()
    src = tmp_path / "src"
    src.mkdir()
    for f in ("pyproject.toml", "setup.py", "README.md"):
        shutil.copy2(os.path.join(ROOT, f), src / f)
    shutil.copytree(os.path.join(ROOT, "include"), src / "include")
    shutil.copytree(os.path.join(ROOT, "icm_gb300"), src / "icm_gb300",
                    ignore=shutil.ignore_patterns("__pycache__"))   # copy2 keeps mtimes: no rebuild
    out = tmp_path / "dist"
    r = subprocess.run([sys.executable, "-m", "pip", "wheel", "--no-deps", "--no-build-isolation", "--no-index",
                        "-w", str(out), str(src)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    wheels = list(out.glob("icm_gb300-*.whl"))
    assert len(wheels) == 1
    names = set(zipfile.ZipFile(wheels[0]).namelist())
    for f in ("icm_gb300/__init__.py", "icm_gb300/_lib.py", "icm_gb300/autograd.py", "icm_gb300/libicm_gb300.so"):
        assert f in names, f
    assert not any(n.startswith("icm_gb300/_build/") or n.startswith("icm_gb300/csrc/") for n in names)
