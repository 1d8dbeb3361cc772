import glob
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")
CASES = os.path.join(GOLDEN, "cases")
REFERENCE_DIR = os.environ.get("MW_REFERENCE_DIR", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (GB300)")


def golden_cases():
    return sorted(os.path.basename(d) for d in glob.glob(os.path.join(CASES, "*")) if os.path.isdir(d))


def load_case(name):
    d = os.path.join(CASES, name)
    with open(os.path.join(d, "golden.json")) as f:
        g = json.load(f)
    return os.path.join(d, "params.txt"), os.path.join(d, "stars.txt"), g


@pytest.fixture(scope="session")
def built_library():
    from milkywayathome_client_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_built():
    from oracle import oracle as orc
    orc.build(reference=os.path.isdir(os.path.join(REFERENCE_DIR, "milkyway_separation")))
    return orc


@pytest.fixture(scope="session")
def gpu_ctx(built_library):
    import milkywayathome_client_gb300 as mw
    ctx = mw.Context(0)
    yield ctx
    ctx.close()
