"""Generate the golden fixtures in tests/golden/ from the AccRQA reference tree.

Run where the reference sources are, named by ACCRQA_REFERENCE_TREE, after
`make -C oracle ref REF=<tree>`, which builds the reference's own CPU code
into oracle/_ref/libaccrqa_ref.so:

    ACCRQA_REFERENCE_TREE=<tree> python tests/golden/make_golden.py

Outputs (all small, committed):
  crqa_input.npy          the 1122-sample series of the reference's CRQA
                          known-answer tests (tests/testthat/testdata/input.txt)
  crqa_kat.json           CRQA values the reference's C++ test holds
                          (tests/test_RQA.cpp:1179-1358), parsed from that file
  r_fixtures.json         expected tables of the reference's R tests
                          (tests/testthat/testdata/expected_*.rds), decoded
  ref_outputs.json        the reference's public CPU API (accrqa_RR/DET/LAM,
                          PLT_CPU) on the CRQA grid, run from oracle/_ref
  ref_histograms.npz      raw RR counts and DET/LAM histograms from the
                          reference's own CPU code on seeded cases (sparse)
"""
from __future__ import annotations

import gzip
import json
import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("ACCRQA_REFERENCE_TREE", "")


# ---------------------------------------------------------------------------
# Minimal reader of R's XDR serialization (enough for data.frames of numeric
# and string columns).
# ---------------------------------------------------------------------------
class _R:
    def __init__(self, data: bytes):
        self.b = data
        self.p = 0
        self.refs = []

    def i32(self):
        v = struct.unpack(">i", self.b[self.p:self.p + 4])[0]
        self.p += 4
        return v

    def length(self):
        n = self.i32()
        if n == -1:
            hi, lo = self.i32(), self.i32()
            n = (hi << 32) + lo
        return n

    def item(self):
        flags = self.i32()
        t = flags & 0xFF
        has_attr = bool(flags & (1 << 9))
        has_tag = bool(flags & (1 << 10))
        if t == 254:                       # NILVALUE
            return None
        if t in (242, 241, 253, 251, 252, 247):
            return None
        if t == 255:                       # REFSXP
            idx = flags >> 8
            if idx == 0:
                idx = self.i32()
            return self.refs[idx - 1]
        if t == 1:                         # SYMSXP
            name = self.item()
            self.refs.append(name)
            return name
        if t == 9:                         # CHARSXP
            n = self.i32()
            if n == -1:
                return None
            s = self.b[self.p:self.p + n].decode("utf-8", "replace")
            self.p += n
            return s
        if t == 2:                         # LISTSXP (pairlist)
            out = {}
            while True:
                attr = self.item() if has_attr else None
                tag = self.item() if has_tag else None
                out[tag] = self.item()
                nxt = self.i32()
                nt = nxt & 0xFF
                if nt == 254:
                    break
                has_attr = bool(nxt & (1 << 9))
                has_tag = bool(nxt & (1 << 10))
                if nt != 2:
                    raise ValueError("unexpected pairlist tail")
            return out
        if t in (10, 13):                  # LGLSXP, INTSXP
            n = self.length()
            v = list(struct.unpack(f">{n}i", self.b[self.p:self.p + 4 * n]))
            self.p += 4 * n
        elif t == 14:                      # REALSXP
            n = self.length()
            v = list(struct.unpack(f">{n}d", self.b[self.p:self.p + 8 * n]))
            self.p += 8 * n
        elif t == 16:                      # STRSXP
            n = self.length()
            v = [self.item() for _ in range(n)]
        elif t == 19:                      # VECSXP
            n = self.length()
            v = [self.item() for _ in range(n)]
        else:
            raise ValueError(f"unsupported SEXP type {t}")
        attrs = self.item() if has_attr else None
        return {"value": v, "attr": attrs}


def read_rds(path):
    raw = open(path, "rb").read()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    r = _R(raw)
    assert r.b[:2] == b"X\n", "only XDR serialization is supported"
    r.p = 2
    ver = r.i32()
    r.i32()
    r.i32()
    if ver == 3:
        n = r.i32()
        r.p += n
    return r.item()


def rds_table(path):
    """A data.frame as {column: list} (numeric columns as floats)."""
    obj = read_rds(path)
    if isinstance(obj, dict) and isinstance(obj.get("value"), list) and obj.get("attr"):
        names = obj["attr"].get("names")["value"]
        cols = {}
        for nm, col in zip(names, obj["value"]):
            cols[nm] = col["value"]
        return cols
    return {"value": obj["value"]}


# ---------------------------------------------------------------------------
def crqa_input():
    txt = open(os.path.join(REF, "tests/testthat/testdata/input.txt")).read().split()
    return np.array([float(v) for v in txt], dtype=np.float64)


def crqa_kat():
    """(tau, emb, lmin/vmin, thr, values...) rows from tests/test_RQA.cpp."""
    src = open(os.path.join(REF, "tests/test_RQA.cpp")).read()
    out = {"DET": {"1": [], "2": []}, "LAM": {"1": [], "2": []}, "RR": {"1": [], "2": []}}
    blocks = {
        "DET": src[src.index("void test_against_CRQA_DET"):src.index("void test_against_CRQA_LAM")],
        "LAM": src[src.index("void test_against_CRQA_LAM"):src.index("void test_against_CRQA_RR")],
        "RR": src[src.index("void test_against_CRQA_RR"):src.index("int main(void)")],
    }
    num = r"([-+0-9.eE]+)"
    for kind, blk in blocks.items():
        dist = "1"
        for line in blk.splitlines():
            if "DST_MAXIMAL" in line:
                dist = "2"
            if not re.search(r"\btau\s*=", line) or "CRQA_" not in line:
                continue
            vals = dict(re.findall(r"(\w+)\s*=\s*" + num, line))
            row = {k: float(v) for k, v in vals.items()}
            out[kind][dist].append(row)
    return out


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "src")):
        raise SystemExit("set ACCRQA_REFERENCE_TREE to the AccRQA reference source tree")
    from oracle import oracle
    oracle.build()
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libaccrqa_ref.so missing: run `make -C oracle ref`")

    x = crqa_input()
    assert len(x) == 1122
    np.save(os.path.join(HERE, "crqa_input.npy"), x)

    kat = crqa_kat()
    json.dump({"source": "tests/test_RQA.cpp:1179-1358 (CRQA known answers, tol 1e-4)",
               "series": "crqa_input.npy", "cases": kat},
              open(os.path.join(HERE, "crqa_kat.json"), "w"), indent=1)

    rfx = {}
    tdir = os.path.join(REF, "tests/testthat/testdata")
    for f in sorted(os.listdir(tdir)):
        if f.startswith("expected_") and f.endswith(".rds"):
            rfx[f[:-4]] = rds_table(os.path.join(tdir, f))
    rin = read_rds(os.path.join(tdir, "input.rds"))["value"]
    assert np.allclose(np.array(rin), x), "input.rds and input.txt differ"
    json.dump({"source": "tests/testthat/testdata/expected_*.rds (CRQA tol 1e-6, PyRQA tol 1e-3)",
               "grid": {"tau": [6, 10], "emb": [3, 4], "thr": [1.2, 1.8], "lmin": 2},
               "tables": rfx}, open(os.path.join(HERE, "r_fixtures.json"), "w"), indent=1)

    # public CPU API of the reference on the CRQA grid
    taus, embs, thr = [6, 10], [3, 4], [1.2, 1.8]
    ref_out = {}
    for dist in (1, 2):
        ref_out[f"RR_{dist}"] = oracle.ref_api_rr(x, taus, embs, thr, dist).tolist()
        for entr in (1, 0):
            ref_out[f"DET_{dist}_{entr}"] = oracle.ref_api_det_lam(
                "DET", x, taus, embs, [2, 3], thr, dist, entr).tolist()
            ref_out[f"LAM_{dist}_{entr}"] = oracle.ref_api_det_lam(
                "LAM", x, taus, embs, [2, 3], thr, dist, entr).tolist()
    json.dump({"source": "reference accrqa_RR/DET/LAM with PLT_CPU (oracle/_ref), "
                         "CPU output order [tau][emb][thr][lmin][5] for DET",
               "taus": taus, "embs": embs, "lmins": [2, 3], "thr": thr, "out": ref_out},
              open(os.path.join(HERE, "ref_outputs.json"), "w"))

    # raw integers from the reference's own CPU code on seeded cases
    from accrqa_gb300 import workloads
    rng = np.random.default_rng(20261203)
    arrays = {}
    cases = []
    gens = [("logistic", workloads.logistic), ("lorenz", workloads.lorenz_x),
            ("white", workloads.white), ("ar1", workloads.ar1)]
    i = 0
    for gname, gen in gens:
        for dt in ("f32", "f64"):
            for dist in (1, 2):
                n = int(rng.integers(60, 420))
                tau = int(rng.integers(1, 5))
                emb = int(rng.integers(1, 9))
                if n - (emb - 1) * tau < 2:
                    emb = 1
                seed = int(rng.integers(0, 1 << 30))
                xs = gen(n, seed).astype(np.float32 if dt == "f32" else np.float64)
                if i % 3 == 0:
                    xs = (np.round(xs * 8) / 8).astype(xs.dtype)   # exact ties
                sd = float(np.std(xs.astype(np.float64)))
                t = (np.array([0.0, 0.1, 0.25, 0.5, 1.0]) * sd).astype(xs.dtype)
                key = f"c{i}"
                arrays[key + "_x"] = xs
                arrays[key + "_thr"] = t
                arrays[key + "_rr"] = oracle.rr_counts(xs, tau, emb, t, dist, use_ref=True)
                det = np.stack([oracle.det_hist(xs, tau, emb, v, dist, use_ref=True) for v in t])
                lam = np.stack([oracle.lam_hist(xs, tau, emb, v, dist, use_ref=True) for v in t])
                arrays[key + "_det"] = det
                arrays[key + "_lam"] = lam
                cases.append({"key": key, "gen": gname, "dtype": dt, "dist": dist, "n": n,
                              "tau": tau, "emb": emb, "seed": seed})
                i += 1
    np.savez_compressed(os.path.join(HERE, "ref_histograms.npz"), **arrays)
    json.dump({"source": "reference CPU code (oracle/_ref): R_matrix_element counts, "
                         "rqa_CPU_DET_metric_parallel_mk1, rqa_CPU_LAM_metric_parallel",
               "cases": cases}, open(os.path.join(HERE, "ref_histograms.json"), "w"), indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
