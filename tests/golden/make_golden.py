#!/usr/bin/env python
"""Regenerates the golden fixtures of this directory from the reference checkout.

Run in a container that has the reference sources (default /root/reference, or
$MHSW_REFERENCE) on x86_64; the GPU machine needs only the committed JSON files.

  ssw_known_answers.json
      The known-answer cases of the reference's unit test test/ssw-test.cpp
      (TEST(MHMTest, ssw), lines 151-238, and the expectations of TEST(MHMTest, AdeptSW),
      lines 241-431), extracted from the test source, plus the outputs of the reference
      SSW (src/ssw/, built by oracle/Makefile) for each case under the three scorings the
      test uses (SSW defaults 2/2/3/1/2, MHM2's ALN_* 1/1/1/1/1, the cigar scoring
      2/4/4/2/1) and the measured scoring 1/3/5/2/2.
  ssw_reference_samples.json
      Seeded sample pairs of the measured workloads and hand-made edge cases with the
      reference SSW's (score, a_begin, a_end, b_begin, b_end) under those four scorings.
  ssw_reference_config0.npz
      The reference SSW's outputs (score, a_begin, a_end, b_begin, b_end,
      sw_score_next_best, ref_end_next_best) for all 10,000 pairs of the 150/300 bp
      workload (workloads.generate(0), regenerated from its seed where the fixture is
      read) at scoring 1/3/5/2/2, from the x86_64 SSE2 build: the record other builds of
      the reference (the aarch64 NEON-shim build) are checked against.
  The two JSON files also record, per scoring, the reference's second-best score and its row
  ("reference_next_best": sw_score_next_best, ref_end_next_best) for maskLen =
  max(len(A)/2, 15) as klign passes it, and what the reference returns with
  report_cigar (Filter(true, true, 0, 32767), the filter klign's post-assembly alignment
  uses): "reference_cigar" = [cigar_string, mismatches].
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

REF = Path(os.environ.get("MHSW_REFERENCE", "/root/reference"))
SCORINGS = {
    "ssw_default": (2, 2, 3, 1, 2),
    "mhm2_aln": (1, 1, 1, 1, 1),
    "cigar": (2, 4, 4, 2, 1),
    "measured": (1, 3, 5, 2, 2),
}


def parse_ssw_test(text: str) -> list[dict]:
    """Walks TEST(MHMTest, ssw) statement by statement, tracking the string variables
    and collecting every check_alns / check_not_alns with the sequences current at the call."""
    body = text[text.index("TEST(MHMTest, ssw)"):text.index("#ifdef ENABLE_GPUS", text.index("TEST(MHMTest, ssw)"))]
    body = re.sub(r"//[^\n]*", "", body)
    vars_: dict[str, str] = {}
    cases = []
    for stmt in body.split(";"):
        stmt = stmt.strip()
        m = re.match(r'^(?:string\s+)?(\w+)\s*=\s*"([ACGTN]*)"$', stmt)
        if m:
            vars_[m.group(1)] = m.group(2)
            continue
        m = re.match(r"^(?:string\s+)?(\w+)\s*=\s*(\w+)$", stmt)
        if m and m.group(2) in vars_:
            vars_[m.group(1)] = vars_[m.group(2)]
            continue
        m = re.match(r'^check_alns\(alns,\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\w+),\s*(\w+),\s*"([^"]*)"\)$',
                     stmt)
        if m:
            q, r = vars_[m.group(6)], vars_[m.group(7)]
            cases.append({"query": q, "ref": r, "qbegin": int(m.group(1)), "qend": int(m.group(2)),
                          "rbegin": int(m.group(3)), "rend": int(m.group(4)), "mismatches": int(m.group(5)),
                          "cigar": m.group(8), "kind": "aln"})
            continue
        m = re.match(r"^check_not_alns\(alns,\s*(\w+),\s*(\w+)\)$", stmt)
        if m:
            cases.append({"query": vars_[m.group(1)], "ref": vars_[m.group(2)], "kind": "no_aln"})
    return cases


def parse_adept_test(text: str) -> list[dict]:
    """Expectations of TEST(MHMTest, AdeptSW): per case ref, query, qstart, qend, rstart, rend."""
    body = re.sub(r"//[^\n]*", "", text[text.index("TEST(MHMTest, AdeptSW)"):])
    vars_: dict[str, str] = {}
    out, cur = [], {}
    for stmt in body.split(";"):
        stmt = stmt.strip()
        m = re.match(r'^(?:string\s+)?(ref|query)\s*=\s*"([ACGTN]*)"$', stmt)
        if m:
            vars_[m.group(1)] = m.group(2)
            continue
        m = re.match(r"^(?:string\s+)?query\s*=\s*ref$", stmt)
        if m:
            vars_["query"] = vars_["ref"]
            continue
        m = re.match(r"^queries\.push_back\(query\)$", stmt)
        if m:
            cur = {"query": vars_["query"], "ref": vars_["ref"]}
            continue
        m = re.match(r"^(qstarts|qends|rstarts|rends)\.push_back\((\d+)\)$", stmt)
        if m and cur:
            cur[m.group(1)[:-1]] = int(m.group(2))
            if len(cur) == 6:
                out.append(cur)
                cur = {}
    return out


def _cigars(oracle, pairs, sc) -> list[list]:
    out, ops, nops = oracle.ref_cigar_batch(pairs, sc, 1, ops_cap=1024)
    assert (nops >= 0).all()
    return [[oracle.cigar_string(ops[i], int(nops[i])), int(out[i, 5])] for i in range(pairs.n)]


def main() -> None:
    from mhm2_staging_gb300 import Pairs, workloads
    from oracle import oracle

    oracle.build(with_reference=True)
    text = (REF / "test" / "ssw-test.cpp").read_text()
    cases = parse_ssw_test(text)
    adept = parse_adept_test(text)
    assert len(cases) == 18, len(cases)
    assert len(adept) == 18, len(adept)
    # A = SSW ref = the test's ref; B = SSW query = the test's query (Align(query, ref))
    pairs = Pairs.from_lists([c["ref"] for c in cases], [c["query"] for c in cases])
    for name, sc in SCORINGS.items():
        out = oracle.ref_align_batch(pairs, sc, 1, score2=True)
        for c, o in zip(cases, out.tolist()):
            c.setdefault("reference", {})[name] = o[:5]
            c.setdefault("reference_next_best", {})[name] = o[5:7]
        for c, cg in zip(cases, _cigars(oracle, pairs, sc)):
            c.setdefault("reference_cigar", {})[name] = cg
    for c, a in zip(cases, adept):
        assert (c["query"], c["ref"]) == (a["query"], a["ref"])
        c["adept_expect"] = {"qbegin": a["qstart"], "qend": a["qend"], "rbegin": a["rstart"], "rend": a["rend"]}
    (HERE / "ssw_known_answers.json").write_text(json.dumps(
        {"source": "test/ssw-test.cpp (TEST(MHMTest, ssw) :151-238; TEST(MHMTest, AdeptSW) :241-431)",
         "orientation": "A = SSW ref = the test's ref; B = SSW query = the test's query",
         "result_layout": "score, a_begin, a_end, b_begin, b_end",
         "scorings": {k: list(v) for k, v in SCORINGS.items()}, "cases": cases}, indent=1))

    # Seeded samples of the measured workloads plus edge cases.
    samples = []
    for cfg, n in ((0, 60), (1, 60), (2, 60), (4, 8)):
        p = workloads.generate(cfg, n=n, first=1000)
        samples += [(f"config{cfg}", p.a(i).decode(), p.b(i).decode()) for i in range(p.n)]
    edge = [
        ("edge", "A", "A"), ("edge", "A", "C"), ("edge", "N", "N"), ("edge", "ACGT", "acgt"),
        ("edge", "UUUU", "AAAA"), ("edge", "NNNNNNNNNN", "ACGTACGTAC"), ("edge", "GATTACA" * 3, "GATTACA"),
        ("edge", "ACGTXYZ-ACGT", "ACGT.ACGT"), ("edge", "T" * 40, "T"), ("edge", "AC" * 60, "CA" * 70),
        ("edge", "ACGTTGCA" * 20, "TGCAACGT" * 25), ("edge", "A" * 300, "A" * 280),
        ("edge", "ACGNNACGT", "ACGTTACGT"), ("edge", "acgtn" * 10, "ACGTN" * 12),
    ]
    samples += edge
    sp = Pairs.from_lists([s[1] for s in samples], [s[2] for s in samples])
    rec = [{"set": s[0], "a": s[1], "b": s[2], "reference": {}, "reference_next_best": {}, "reference_cigar": {}}
           for s in samples]
    for name, sc in SCORINGS.items():
        out = oracle.ref_align_batch(sp, sc, 1, score2=True)
        for r, o in zip(rec, out.tolist()):
            r["reference"][name] = o[:5]
            r["reference_next_best"][name] = o[5:7]
        for r, cg in zip(rec, _cigars(oracle, sp, sc)):
            r["reference_cigar"][name] = cg
    (HERE / "ssw_reference_samples.json").write_text(json.dumps(
        {"source": "reference SSW (src/ssw/ssw.cpp + ssw_core.cpp) called as klign calls it (src/klign.cpp:257)",
         "orientation": "a = SSW ref (klign: the read), b = SSW query (klign: the contig window)",
         "result_layout": "score, a_begin, a_end, b_begin, b_end",
         "scorings": {k: list(v) for k, v in SCORINGS.items()}, "pairs": rec}))
    print(f"{len(cases)} known-answer cases, {len(rec)} sample pairs")
    make_protein(oracle, Pairs)


def make_protein(oracle, Pairs) -> None:
    """ssw_protein_samples.json: seeded protein pairs (random, and mutated copies with
    indels and flanks) with a seeded symmetric 24 x 24 matrix (diagonal 4..11, elsewhere
    -4..3) and the 24-letter encoding, and the reference SSW's outputs (Aligner with that
    matrix and translation, SetGapPenalty) under three gap settings."""
    import numpy as np

    rng = np.random.default_rng(2024)
    m = rng.integers(-4, 4, (24, 24))
    m = np.triu(m) + np.triu(m, 1).T
    np.fill_diagonal(m, rng.integers(4, 12, 24))
    enc = oracle.protein_encoding()
    letters = oracle.PROTEIN_LETTERS
    a, b = [], []
    for k in range(240):
        x = "".join(rng.choice(list(letters[:20]) + ["B", "Z", "X", "*"], rng.integers(1, 600)))
        if k % 4 == 0:
            y = "".join(rng.choice(list(letters), rng.integers(1, 500)))
        else:
            y = []
            for ch in x:
                r = rng.random()
                if r < 0.03:
                    continue
                if r < 0.06:
                    y.append("".join(rng.choice(list(letters[:20]), rng.integers(1, 4))))
                y.append(ch if rng.random() > 0.15 else rng.choice(list(letters)))
            y = "".join(rng.choice(list(letters[:20]), rng.integers(0, 50))) + "".join(y) + "A"
        a.append(x)
        b.append(y)
    pairs = Pairs.from_lists(a, b)
    gaps = [[11, 1], [10, 2], [5, 2]]
    rec = {"matrix": m.astype(int).tolist(), "encoding": enc.astype(int).tolist(), "gaps": gaps,
           "pairs": [{"a": x, "b": y} for x, y in zip(a, b)]}
    for go, ge in gaps:
        out = oracle.ref_protein_batch(pairs, m.astype(np.int16), enc, go, ge)
        for r, o in zip(rec["pairs"], out.tolist()):
            r.setdefault("reference", {})[f"{go}/{ge}"] = o
    rec["source"] = ("reference SSW (src/ssw) as Aligner(matrix, 24, translation, 128) + SetGapPenalty; "
                     "A = SSW ref, B = SSW query")
    (HERE / "ssw_protein_samples.json").write_text(json.dumps(rec))
    print(f"{len(a)} protein pairs")


def make_config0(oracle) -> None:
    import numpy as np

    from mhm2_staging_gb300 import workloads

    oracle.build(with_reference=True)
    pairs = workloads.generate(0)
    out = oracle.ref_align_batch(pairs, SCORINGS["measured"], score2=True)
    np.savez_compressed(HERE / "ssw_reference_config0.npz", out=out.astype(np.int32),
                        scoring=np.array(SCORINGS["measured"], dtype=np.int32))
    print(f"config 0: {pairs.n} pairs")


if __name__ == "__main__":
    from oracle import oracle as _oracle

    if sys.argv[1:] == ["config0"]:
        make_config0(_oracle)
    else:
        main()
        make_config0(_oracle)
