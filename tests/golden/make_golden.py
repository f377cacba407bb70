"""Generate the golden fixtures under tests/golden/ (run in a container that
has the reference tree; the fixtures are committed and the tests only read
them).

* saber_gb300/data/karlin.json — the NCBI blast_stat.c gapped
  Karlin-Altschul tables as listed in src/scoring/stats.rs.
* defects.json — the reference's defect-reproduction inputs
  (bench/defects/*.fa) and the outputs its v1.2.0 binary recorded for them
  (bench/results/v1.2.0/defects.json).
* matrices.json — the substitution tables of src/scoring/matrices.rs (the
  public NCBI BLOSUM/PAM tables in NCBI order ARNDCQEGHILKMFPSTWYVBZX*),
  parsed from the reference source; also copied to saber_gb300/data/.
* sw_vectors.json — the test vectors of examples/gpu_vectors.rs (same
  xorshift generator, seed 0xC0DA, same case mix), with expected scores
  computed by the reference's own CUDA kernel source (src/gpu/kernels/sw.cu)
  compiled for the host by oracle/Makefile (`make -C oracle ref`).

Usage:  python tests/golden/make_golden.py --ref-root <reference checkout>
        (or SABER_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py)
"""
import argparse
import ctypes
import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

NAMES = {
    "BLOSUM45_MATRIX": "BLOSUM45", "BLOSUM50_MATRIX": "BLOSUM50",
    "BLOSUM62_MATRIX": "BLOSUM62", "BLOSUM80_MATRIX": "BLOSUM80",
    "BLOSUM90_MATRIX": "BLOSUM90", "PAM30_MATRIX": "PAM30",
    "PAM70_MATRIX": "PAM70", "PAM250_MATRIX": "PAM250",
}


def parse_matrices(ref_root):
    src = open(os.path.join(ref_root, "src/scoring/matrices.rs")).read()
    out = {}
    for const, name in NAMES.items():
        m = re.search(r"const %s: \[\[i32; 24\]; 24\] = \[(.*?)\n\];" % const, src, re.S)
        if not m:
            raise SystemExit("matrix %s not found" % const)
        rows = re.findall(r"\[([^\[\]]+)\]", m.group(1))
        mat = [[int(v) for v in r.split(",") if v.strip()] for r in rows]
        assert len(mat) == 24 and all(len(r) == 24 for r in mat), name
        out[name] = mat
    return out


def parse_karlin(ref_root):
    """The NCBI blast_stat.c Karlin-Altschul tables of src/scoring/stats.rs:
    rows (existence, extension, lambda, K, H, alpha, beta)."""
    src = open(os.path.join(ref_root, "src/scoring/stats.rs")).read()
    row = r"Row\(\s*(-?\d+),\s*(-?\d+),\s*([-\d.eE]+),\s*([-\d.eE]+),\s*([-\d.eE]+),\s*([-\d.eE]+),\s*([-\d.eE]+)\)"
    out = {"protein": {}, "nucleotide": []}
    for name in NAMES.values():
        u = re.search(r"const UNGAPPED_%s: Row = %s;" % (name, row), src)
        t = re.search(r"const %s: &\[Row\] = &\[(.*?)\];" % name, src, re.S)
        rows = [[int(m[0]), int(m[1])] + [float(x) for x in m[2:]] for m in re.findall(row, t.group(1))]
        out["protein"][name] = {"ungapped": [int(u.group(1)), int(u.group(2))] + [float(u.group(k)) for k in range(3, 8)],
                                "gapped": rows}
    nt = re.search(r"const NT_TABLES: &\[NtTable\] = &\[(.*?)\n\];", src, re.S).group(1)
    for m in re.finditer(r"NtTable \{ reward: (-?\d+), penalty: (-?\d+), even_only: (true|false), rows: &\[(.*?)\] \}",
                         nt, re.S):
        rows = [[int(x[0]), int(x[1])] + [float(y) for y in x[2:]] for x in re.findall(row, m.group(4))]
        out["nucleotide"].append({"reward": int(m.group(1)), "penalty": int(m.group(2)),
                                  "even_only": m.group(3) == "true", "rows": rows})
    return out


def read_fasta(path):
    recs, name, seq = [], None, []
    for line in open(path):
        line = line.strip()
        if line.startswith(">"):
            if name is not None:
                recs.append((name, "".join(seq)))
            name, seq = line[1:].split()[0], []
        elif line:
            seq.append(line)
    if name is not None:
        recs.append((name, "".join(seq)))
    return recs


def defect_cases(ref_root):
    """bench/defects/*.fa with the outputs the reference binary (v1.2.0)
    recorded for them in bench/results/v1.2.0/defects.json."""
    rec = json.load(open(os.path.join(ref_root, "bench/results/v1.2.0/defects.json")))
    out = []
    for name in ("gap", "amb", "amb2", "long", "sat"):
        q = read_fasta(os.path.join(ref_root, "bench/defects/%s_q.fa" % name))
        d = read_fasta(os.path.join(ref_root, "bench/defects/%s_db.fa" % name))
        runs = {k: v for k, v in rec[name].items() if k.startswith("v1.2.0") and "score" in v}
        out.append({"name": name, "query": q, "db": d, "recorded": runs})
    return out


def nucleotide(match, mismatch):
    # matrices.rs:85-91
    mat = [[mismatch] * 24 for _ in range(24)]
    for i in range(4):
        mat[i][i] = match
    return mat


class XorShift:
    """examples/gpu_vectors.rs:10-21"""

    def __init__(self, seed):
        self.s = seed

    def next(self):
        s = self.s
        s ^= (s << 13) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 7
        s ^= (s << 17) & 0xFFFFFFFFFFFFFFFF
        self.s = s
        return s

    def below(self, n):
        return self.next() % n


def gpu_vector_cases(mats):
    """examples/gpu_vectors.rs:52-90"""
    r = XorShift(0xC0DA)
    blosum, pam, nt = mats["BLOSUM62"], mats["PAM30"], nucleotide(2, -3)
    cases = []
    for case in range(24):
        m, mname, alpha, go, ge = [
            (blosum, "BLOSUM62", 24, 11, 1), (pam, "PAM30", 20, 10, 1),
            (nt, "NT_2_-3", 5, 7, 2), (blosum, "BLOSUM62", 24, 13, 2)][case % 4]
        ql = 1 + r.below(300)
        q = [r.below(alpha) for _ in range(ql)]
        bias = [r.below(5) - 2 for _ in range(ql)] if case % 3 == 0 else None
        nw = 1 + r.below(40)
        wins = []
        for k in range(nw):
            if k % 5 == 0:
                lo = r.below(ql)
                hi = lo + r.below(ql - lo + 1)
                w = []
                for c in q[lo:hi]:
                    if r.below(4) == 0:
                        w.append(r.below(alpha))
                    else:
                        w.append(c)
                wins.append(w)
            else:
                l = r.below(400)
                wins.append([r.below(alpha) for _ in range(l)])
        cases.append(dict(matrix=mname, gap_open=go, gap_extend=ge, query=q, bias=bias, windows=wins))
    long = [17] * 4000
    cases.append(dict(matrix="BLOSUM62", gap_open=11, gap_extend=1, query=long, bias=None,
                      windows=[long, long[:3500]]))
    cases.append(dict(matrix="BLOSUM62", gap_open=11, gap_extend=1, query=[0, 1, 2, 200, 4],
                      bias=None, windows=[[0, 1, 2, 22, 4], [255, 255]]))
    return cases


def ref_scores(lib, case, mats):
    mat = mats[case["matrix"]] if case["matrix"] in mats else nucleotide(2, -3)
    flat = (ctypes.c_int32 * 576)(*[v for row in mat for v in row])
    q = bytes(case["query"])
    bias = case["bias"]
    cb = (ctypes.c_int8 * len(bias))(*bias) if bias else None
    subj = b"".join(bytes(w) for w in case["windows"])
    offs = [0]
    for w in case["windows"]:
        offs.append(offs[-1] + len(w))
    coffs = (ctypes.c_uint32 * len(offs))(*offs)
    out = (ctypes.c_int32 * len(case["windows"]))()
    lib.ref_sw_score_windows(q, len(q), cb, subj if subj else None, coffs, len(case["windows"]),
                             flat, case["gap_open"], case["gap_extend"], out)
    return list(out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("SABER_REFERENCE_ROOT"),
                    help="the reference checkout (default: $SABER_REFERENCE_ROOT)")
    a = ap.parse_args()
    if not a.ref_root:
        ap.error("give --ref-root or set SABER_REFERENCE_ROOT to the reference checkout")
    mats = parse_matrices(a.ref_root)
    with open(os.path.join(HERE, "matrices.json"), "w") as f:
        json.dump(mats, f)
    data_dir = os.path.join(REPO, "saber_gb300", "data")
    os.makedirs(data_dir, exist_ok=True)
    shutil.copy(os.path.join(HERE, "matrices.json"), os.path.join(data_dir, "matrices.json"))
    with open(os.path.join(data_dir, "karlin.json"), "w") as f:
        json.dump(parse_karlin(a.ref_root), f)

    with open(os.path.join(HERE, "defects.json"), "w") as f:
        json.dump({"source": "bench/defects/*.fa and bench/results/v1.2.0/defects.json", "cases": defect_cases(a.ref_root)},
                  f, indent=0)

    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref",
                           "REF_ROOT=%s" % a.ref_root])
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libref_sw.so"))
    cases = gpu_vector_cases(mats)
    for c in cases:
        c["expected"] = ref_scores(lib, c, mats)
    with open(os.path.join(HERE, "sw_vectors.json"), "w") as f:
        json.dump({"source": "examples/gpu_vectors.rs generator; scores from src/gpu/kernels/sw.cu "
                             "compiled for the host (oracle/_ref)", "cases": cases}, f)
    n = sum(len(c["windows"]) for c in cases)
    print("wrote %d cases, %d windows" % (len(cases), n), file=sys.stderr)


if __name__ == "__main__":
    main()
