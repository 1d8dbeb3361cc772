"""The C-ABI library: it loads, it exports every function the header
declares, its struct layouts match the header (and the reference's), and
without an sm_103 GPU it fails loudly instead of falling back."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "milkyway_separation_gb300.h")
TEST_HEADER = os.path.join(REPO, "include", "milkyway_separation_gb300_test.h")


def _functions_in(path):
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    return set(re.findall(r"\b(mwsep_\w+)\s*\(", text))


def _declared_functions():
    """Every function the library's headers declare: the product ABI and the
    test/diagnostic entry points."""
    return sorted(_functions_in(HEADER) | _functions_in(TEST_HEADER))


def test_public_header_holds_no_test_entry_points():
    """The product header declares the evaluator ABI only; the debug-build
    checks, primitive probes and launch-model diagnostics live in the test
    header."""
    test_only = _functions_in(TEST_HEADER)
    assert test_only == {"mwsep_device_checks", "mwsep_df_eval", "mwsep_log10_sum_eval", "mwsep_model_tile_cost",
                         "mwsep_model_kchunk"}
    assert not (test_only & _functions_in(HEADER))


def test_library_exports_every_declared_function(built_library):
    lib = ctypes.CDLL(built_library)
    names = _declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_library):
    from milkywayathome_client_gb300 import native
    assert set(_declared_functions()) <= set(native.exported_symbols())


def _prototype_arg_counts():
    """name -> number of parameters, from the header's prototypes."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read() + open(TEST_HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(mwsep_\w+)\s*\(([^;{]*?)\)\s*;", text):
        args = m.group(2).strip()
        depth, n = 0, (0 if args in ("", "void") else 1)
        for ch in args:
            depth += ch == "("
            depth -= ch == ")"
            n += ch == "," and depth == 0
        out[m.group(1)] = n
    return out


def test_python_binding_argument_counts(built_library):
    """Each ctypes signature has as many arguments as the header's prototype."""
    from milkywayathome_client_gb300 import native
    protos = _prototype_arg_counts()
    assert set(protos) == set(_declared_functions())  # every declared function parsed
    wrong = {n: (protos[n], len(native._SIGS[n][1])) for n in protos
             if n in native._SIGS and protos[n] != len(native._SIGS[n][1])}
    assert not wrong, wrong


def test_struct_layouts_match_c(tmp_path, built_library):
    """sizeof/offsetof from a C compiler vs the ctypes mirror."""
    from milkywayathome_client_gb300 import native as N
    structs = {
        "INTEGRAL": N.INTEGRAL, "ASTRONOMY_PARAMETERS": N.ASTRONOMY_PARAMETERS, "STAR_POINTS": N.STAR_POINTS,
        "INTEGRAL_AREA": N.INTEGRAL_AREA, "EVALUATION_STATE": N.EVALUATION_STATE, "mwsep_result": N.mwsep_result,
        "mwsep_pipe_peaks": N.mwsep_pipe_peaks, "mwsep_area_tables": N.mwsep_area_tables,
        "mwsep_density_params": N.mwsep_density_params, "mwsep_request": N.mwsep_request,
        "mwsep_server_config": N.mwsep_server_config, "mwsep_server_stats": N.mwsep_server_stats,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(out[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"


def test_header_compiles_after_reference_headers(tmp_path):
    """The reference's own headers and this header can share a translation
    unit: the structs are guarded by the reference include guards."""
    ref = os.environ.get("MW_REFERENCE_DIR", "/root/reference")
    cpu = os.path.join(ref, "milkyway_separation", "cpu")
    if not os.path.isdir(cpu):
        pytest.skip("reference sources not present")
    src = tmp_path / "both.c"
    src.write_text(f'#include "parameters.h"\n#include "star_points.h"\n#include "evaluation_state.h"\n'
                   f'#include "simple_evaluator.h"\n#include "{HEADER}"\n'
                   "EvalFunc f = mwsep_evaluate;\nint main(void){return f == 0;}\n")
    subprocess.run(["gcc", "-std=gnu99", "-c", "-o", str(tmp_path / "both.o"), "-I", cpu, str(src)], check=True)


def _has_sm103():
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=compute_cap", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30)
        return out.returncode == 0 and "10.3" in out.stdout
    except Exception:
        return False


@pytest.mark.skipif(_has_sm103(), reason="a GB300 is present; this checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(built_library):
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    with pytest.raises(mw.MwsepError) as e:
        mw.Context(0)
    assert e.value.status == N.MWSEP_ERR_CUDA
