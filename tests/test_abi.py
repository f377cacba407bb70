"""CPU tests of the C-ABI boundary: the library loads, exports every symbol
declared in include/*.h, the header carries no framework types, and the
host-only helpers work without a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300 import gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(saber_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = _declared()
    for want in ("saber_gpu_open", "saber_gpu_close", "saber_gpu_score_band_jobs", "saber_gpu_score_windows",
                 "saber_gpu_score_banded_many", "saber_band_cells"):
        assert want in names


def test_headers_use_plain_c_types():
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        assert "torch" not in src and "at::" not in src and "std::" not in src


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(gpu.lib_path())
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_band_cells_matches_oracle_cell_count():
    rng = np.random.default_rng(11)
    from saber_gb300.scoring import matrix
    mat = matrix("BLOSUM62")
    for _ in range(300):
        m = int(rng.integers(1, 60))
        n = int(rng.integers(1, 60))
        lo = int(rng.integers(-80, 80))
        hi = lo + int(rng.integers(-5, 90))
        q = rng.integers(0, 20, m).astype(np.uint8)
        s = rng.integers(0, 20, n).astype(np.uint8)
        want = orc.banded_score(q, s, None, mat, 11, 1, lo, hi)[3]
        assert gpu.band_cells(m, n, lo, hi) == want, (m, n, lo, hi)


def test_open_without_gpu_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu.SaberGpuError):
        gpu.Device(0)


def test_headers_compile_as_plain_c(tmp_path):
    """The boundary is plain C: every header compiles as C99 on its own and
    a C translation unit can call through it."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c", h],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    src = tmp_path / "use.c"
    src.write_text('#include "saber_gpu.h"\nint main(void) { saber_gpu* h = 0; saber_tantan_params p = {0};\n'
                   '  (void)p; return saber_gpu_open(0, &h); }\n')
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(REPO, "include"), "-c", str(src), "-o",
                        str(tmp_path / "use.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ctypes_mirrors_match_the_header(tmp_path):
    """Every ctypes mirror of a header struct has the C struct's size and
    field offsets (compiled against include/saber_gpu.h)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"saber_score_stats": gpu.ScoreStats, "saber_scan_params": gpu.ScanParams,
             "saber_scan_stats": gpu.ScanStats, "saber_alignment": gpu.Alignment,
             "saber_traceback_stats": gpu.TracebackStats, "saber_search_params": gpu.SearchParamsC,
             "saber_search_stats": gpu.SearchStats, "saber_triage_train_cfg": gpu.TriageTrainCfg,
             "saber_triage_train_stats": gpu.TriageTrainStats}
    cfield = {"lambda_": "lambda"}  # Python keyword
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "saber_gpu.h"', 'int main(void) {']
    for cname, py in pairs.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, cfield.get(f, f)))
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for cname, py in pairs.items():
        assert int(out[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[cname + "." + f]) == getattr(py, f).offset, (cname, f)
