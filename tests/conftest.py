"""Shared fixtures.  ``-m gpu`` tests need a CUDA device and the built library; the
rest run on CPU (oracle against the golden fixtures, deck parsing, C-ABI exports)."""
import importlib
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
if os.path.join(ROOT, "tests") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libthesis_gb300.so")


@pytest.fixture(scope="session")
def thesis():
    return importlib.import_module("3dthesis_gb300")


@pytest.fixture(scope="session")
def decks():
    return importlib.import_module("3dthesis_gb300.decks")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def deck_dir(tmp_path_factory, decks):
    """Writes a named deck once per session; returns the ParamInput.txt path."""
    base = tmp_path_factory.mktemp("decks")
    made = {}

    def make(name, *args, mutate=None, tag=None):
        key = tag or (name + "_" + "_".join(map(str, args)))
        if key not in made:
            d = getattr(decks, name)(*args)
            if mutate:
                mutate(d)
            made[key] = d.write(str(base / key))
        return made[key]
    return make


@pytest.fixture(scope="session")
def built_library(thesis):
    lib = thesis.LIB_PATH
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    return lib
