"""Shared fixtures: the product package, the CPU restatement (checker), the
reference's golden files."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on the device)")


@pytest.fixture(scope="session")
def tp():
    lib = os.path.join(graft.PKG_DIR, "libtp_gb300.so")
    if not os.path.exists(lib):
        graft.build()
    return graft.package()


@pytest.fixture(scope="session")
def oracle(tp):
    import tp_oracle_py

    if not os.path.exists(tp_oracle_py.LIB) or not os.path.exists(tp_oracle_py.CLI):
        tp_oracle_py.build()
    return tp_oracle_py.Oracle(tp)


@pytest.fixture(scope="session")
def valeurs():
    return os.path.join(GOLDEN, "valeurs")


@pytest.fixture(scope="session")
def cfg_valeurs(oracle, valeurs):
    st, cfg, _ = oracle.load(valeurs)
    assert st == 0
    return cfg


@pytest.fixture(scope="session")
def cfg_sqrts1000(oracle):
    st, cfg, _ = oracle.load(os.path.join(GOLDEN, "valeurs_sqrts1000"))
    assert st == 0
    return cfg


@pytest.fixture(scope="session")
def ctx(tp):
    c = tp.Context(0)
    yield c
    c.close()


def golden(kind, features):
    name = "%s-features_%s" % (kind, features.replace(",", "+") or "default")
    with open(os.path.join(GOLDEN, name)) as fh:
        return fh.read()
