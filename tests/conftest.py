"""Shared pytest setup: the ``gpu`` marker and import paths for the oracle and the package."""
import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / 'cfd-cylinder-flow-ghost-cell_gb300'
PKG_NAME = 'cfd_cylinder_flow_ghost_cell_gb300'
for extra in (ROOT / 'oracle', ROOT):
    if str(extra) not in sys.path:
        sys.path.insert(0, str(extra))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


def load_package():
    """Import the package directory (its name has dashes) under an importable alias."""
    if PKG_NAME in sys.modules:
        return sys.modules[PKG_NAME]
    spec = importlib.util.spec_from_file_location(PKG_NAME, PKG_DIR / '__init__.py',
                                                  submodule_search_locations=[str(PKG_DIR)])
    module = importlib.util.module_from_spec(spec)
    sys.modules[PKG_NAME] = module
    spec.loader.exec_module(module)
    return module


def load_module(name):
    """A submodule of the package (imported through load_package)."""
    load_package()
    return importlib.import_module(f'{PKG_NAME}.{name}')


@pytest.fixture(scope='session')
def pkg():
    return load_package()


GOLDEN = ROOT / 'tests' / 'golden'
