"""Packaging of the GB300 RQA engine.

    pip install .            (or: pip wheel . --no-build-isolation)

builds ``libaccrqa.so`` for sm_103a with nvcc (``accrqa_gb300/build.py``, no
cmake) and installs the ``accrqa_gb300`` package with the library inside it.
The reference's own Python package then runs on it unchanged with
``ACCRQA_LIB_DIR=<site-packages>/accrqa_gb300/lib``.
"""
import importlib.util
import os

from setuptools import setup
from setuptools.command.build_py import build_py
from setuptools.dist import Distribution

HERE = os.path.dirname(os.path.abspath(__file__))


class build_py_with_engine(build_py):
    """Compile the CUDA/C++ library before the package files are collected."""

    def run(self):
        spec = importlib.util.spec_from_file_location(
            "_accrqa_gb300_build", os.path.join(HERE, "accrqa_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        super().run()


class BinaryDistribution(Distribution):
    """The package carries a native library: platform-specific wheels."""

    def has_ext_modules(self):
        return True


setup(
    name="accrqa-gb300",
    version="0.1.0",
    description="GB300-native recurrence quantification analysis behind the AccRQA API",
    packages=["accrqa_gb300"],
    package_data={"accrqa_gb300": ["lib/libaccrqa.so"]},
    python_requires=">=3.10",
    install_requires=["numpy"],
    cmdclass={"build_py": build_py_with_engine},
    distclass=BinaryDistribution,
)
