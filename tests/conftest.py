import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(TESTS, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA engine")


@pytest.fixture(scope="session")
def native():
    """Native library built in-tree and physics data staged."""
    from ompmc_gb300 import _native, build, data

    build.build()
    data.stage()
    return _native.lib()


@pytest.fixture(scope="session")
def oracle(native):
    from oracle import binding

    binding.build()
    binding.lib()
    return binding


@pytest.fixture(scope="session")
def case_dir(tmp_path_factory, native):
    return str(tmp_path_factory.mktemp("cases"))


@pytest.fixture(scope="session")
def problem_factory(case_dir, native):
    from cases import write_case

    from ompmc_gb300 import api

    cache = {}

    def make(name, ncase=None, nbatch=10, seeds=(97, 33)):
        key = (name, ncase, nbatch, seeds)
        if key not in cache:
            d = os.path.join(case_dir, f"{name}_{ncase}_{nbatch}_{seeds[0]}_{seeds[1]}")
            cache[key] = api.Problem.from_file(write_case(name, d, ncase=ncase, nbatch=nbatch, seeds=seeds))
        return cache[key]

    return make


@pytest.fixture(scope="session")
def engine(native):
    from ompmc_gb300 import api

    e = api.Engine(0)
    yield e
    e.close()
