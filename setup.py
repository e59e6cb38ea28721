"""Packaging hook: `pip install .` (or `pip wheel .`) compiles
libicm_gb300.so with nvcc for sm_103a (icm_gb300/build.py) before the
package files are collected, so the wheel carries the library beside the
Python package.  Metadata lives in pyproject.toml."""
import importlib.util
import os

from setuptools import setup
from setuptools.command.build_py import build_py

HERE = os.path.dirname(os.path.abspath(__file__))


class BuildWithLibrary(build_py):
    def run(self):
        # build.py by path: importing the package would load the library
        spec = importlib.util.spec_from_file_location("_icm_gb300_build", os.path.join(HERE, "icm_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        super().run()


setup(cmdclass={"build_py": BuildWithLibrary})
