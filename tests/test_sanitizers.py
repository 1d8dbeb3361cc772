"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (no GPU):
the library's host-only units (I/O, binary formats, finite-difference
consumers, matrix inversion) through tests/sanitize_harness.cpp, and the
oracle restatement through its command-line driver, which must also print
the same numbers as its normal build."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO, load_case

CSRC = os.path.join(REPO, "milkywayathome_client_gb300", "csrc")
SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=undefined", "-g", "-O1"]
CASES = ["basic_1stream", "three_streams", "cut_area", "aux_profile", "sgr_coordinates", "six_streams",
         "single_cell_single_star", "ragged_sizes", "stream_off", "general_alpha_delta"]


def _have(tool):
    return shutil.which(tool) is not None


def _sanitizers_work(tmp_path):
    src = tmp_path / "t.c"
    src.write_text("int main(void){return 0;}\n")
    r = subprocess.run(["gcc", *SAN, str(src), "-o", str(tmp_path / "t")], capture_output=True)
    return r.returncode == 0 and subprocess.run([str(tmp_path / "t")]).returncode == 0


@pytest.fixture(scope="module")
def san_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("san")
    if not (_have("gcc") and _have("g++")) or not _sanitizers_work(d):
        pytest.skip("gcc sanitizers unavailable")
    return d


def _env():
    return dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")


def test_host_units_under_sanitizers(san_dir):
    exe = san_dir / "harness"
    cmd = ["g++", "-std=c++17", *SAN, "-I", os.path.join(REPO, "include"), "-I", CSRC,
           os.path.join(REPO, "tests", "sanitize_harness.cpp"), os.path.join(CSRC, "mwsep_io.cpp"),
           os.path.join(CSRC, "mwsep_binary.cpp"), os.path.join(CSRC, "mwsep_optimise.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    args = []
    for name in CASES:
        pf, sf, _ = load_case(name)
        args += [pf, sf]
    work = san_dir / "work"
    work.mkdir(exist_ok=True)
    r = subprocess.run([str(exe), str(work), *args], capture_output=True, text=True, env=_env(), timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "sanitize harness: ok" in r.stdout
    assert "runtime error" not in r.stderr and "ERROR: AddressSanitizer" not in r.stderr


def test_oracle_under_sanitizers(san_dir, oracle_built):
    exe = san_dir / "sep_oracle_san"
    src = os.path.join(REPO, "oracle", "sep_oracle.c")
    r = subprocess.run(["gcc", "-std=gnu99", "-ffp-contract=off", *SAN, "-DSEP_ORACLE_MAIN", src, "-o", str(exe),
                        "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    plain = os.path.join(REPO, "oracle", "_build", "sep_oracle")
    for name in ["basic_1stream", "cut_area", "aux_profile", "sgr_coordinates", "single_cell_single_star"]:
        pf, sf, g = load_case(name)
        theta = [repr(float(x)) for x in g["theta"]]
        a = subprocess.run([str(exe), "-a", pf, "-p", sf, *theta], capture_output=True, text=True, env=_env(),
                           timeout=600)
        b = subprocess.run([plain, "-a", pf, "-p", sf, *theta], capture_output=True, text=True, timeout=600)
        assert a.returncode == 0, a.stderr
        assert "runtime error" not in a.stderr and "ERROR: AddressSanitizer" not in a.stderr, a.stderr
        assert a.stdout == b.stdout, name
