"""Shared pytest setup.

Markers: ``gpu`` = needs a CUDA device (run on the GB300 machine); everything else runs on CPU.
The oracle (a CPU restatement of Ferrite.jl's assembly path) and the package live in
directories that are not Python packages by name (``oracle/``, ``ferrite.jl_gb300/``);
they are put on ``sys.path`` here.
"""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def load_package():
    """Import ferrite.jl_gb300/ as the module ``ferrite_gb300``."""
    if "ferrite_gb300" in sys.modules:
        return sys.modules["ferrite_gb300"]
    path = os.path.join(ROOT, "ferrite.jl_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location("ferrite_gb300", path,
                                                  submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ferrite_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def fg():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O
