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


REF_FIXTURES = os.path.join(GOLDEN, "reference")
SCALE = os.path.join(GOLDEN, "scale")


def reference_fixture_ids():
    """The reference's own test fixtures that have goldens (79, 86, 11, 12,
    20, 21 and the -aux variants)."""
    with open(os.path.join(REF_FIXTURES, "index.json")) as f:
        return list(json.load(f))


def large_fixture_ids():
    """The reference's large test fixtures (1600 x 640 x 1400 cells: 79, 86,
    12 and the -aux files of 79, 86, 11, 12) that have goldens."""
    d = os.path.join(GOLDEN, "reference_large")
    if not os.path.isdir(d):
        return []
    return sorted(x for x in os.listdir(d) if os.path.exists(os.path.join(d, x, "golden.json")))


def _unpacked(xz_path, tmp_root):
    """The decompressed star file of a committed .xz fixture (once per session)."""
    import lzma
    import shutil
    out = os.path.join(tmp_root, os.path.relpath(xz_path, GOLDEN).replace(os.sep, "_")[: -len(".xz")])
    if not os.path.exists(out):
        with lzma.open(xz_path, "rb") as f, open(out + ".part", "wb") as g:
            shutil.copyfileobj(f, g)
        os.replace(out + ".part", out)
    return out


@pytest.fixture(scope="session")
def golden_inputs(tmp_path_factory):
    """Paths of the committed large fixtures: fn(kind, name) -> (params,
    stars, golden) with kind "reference" (a reference test fixture),
    "reference_large" (one of its large fixtures) or "scale" (a benchmark
    config, name "config1" / "config2")."""
    root = str(tmp_path_factory.mktemp("golden_stars"))

    def get(kind, name):
        if kind in ("reference", "reference_large"):
            d = os.path.join(GOLDEN, kind, name)
            with open(os.path.join(d, "golden.json")) as f:
                g = json.load(f)
            xz = os.path.join(GOLDEN, g["stars_xz"])
        else:
            d = os.path.join(SCALE, name)
            with open(os.path.join(d, "golden.json")) as f:
                g = json.load(f)
            xz = os.path.join(d, "stars.txt.xz")
        return os.path.join(d, "params.txt"), _unpacked(xz, root), g

    return get


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
