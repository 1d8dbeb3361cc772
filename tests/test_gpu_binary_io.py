"""A catalogue loaded from its binary form evaluates to the same bits as the
reference's text star file."""
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["three_streams", "cut_area", "config0"])
def test_binary_catalogue_gives_identical_results(gpu_ctx, tmp_path, name):
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    bp = str(tmp_path / "p.mwsp")
    ap.write_binary(bp)
    cat = str(tmp_path / "s.mwsb")
    mw.StarPoints.read(sf).write_binary(cat)
    out = {}
    for kind, (params, stars) in {"text": (pf, sf), "binary": (bp, cat)}.items():
        a = mw.AstronomyParameters.read(params) if kind == "text" else mw.AstronomyParameters.read_binary(params)
        gpu_ctx.set_problem(a)
        gpu_ctx.set_stars_file(stars)
        out[kind] = [gpu_ctx.evaluate(g["theta"], prec) for prec in (mw.MWSEP_PLAIN_F64, mw.MWSEP_MIXED_F32)]
    for t, b in zip(out["text"], out["binary"]):
        assert t.likelihood == b.likelihood
        assert t.integrals == b.integrals
        assert t.prob_sum == b.prob_sum


def test_c_client_reads_binary_files(built_library, tmp_path):
    """The C client takes the binary forms in place of the text files and
    prints the same result lines."""
    import subprocess
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import build
    pf, sf, g = load_case("three_streams")
    bp, bs = str(tmp_path / "p.mwsp"), str(tmp_path / "s.mwsb")
    mw.AstronomyParameters.read(pf).write_binary(bp)
    mw.StarPoints.read(sf).write_binary(bs)
    theta = [repr(float(x)) for x in g["theta"]]
    outs = []
    for a, p in ((pf, sf), (bp, bs)):
        r = subprocess.run([build.CLIENT_PATH, "-a", a, "-p", p, *theta], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append([ln for ln in r.stderr.splitlines() if ln.startswith("<") and "seconds" not in ln
                     and "search_application" not in ln])
    assert outs[0] == outs[1] and len(outs[0]) >= 3
