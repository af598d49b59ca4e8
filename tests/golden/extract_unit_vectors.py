#!/usr/bin/env python3
"""Extract the reference's own unit-test vectors into tests/golden/unit_vectors.json.

The reference keeps exact expected results for the pieces of its mapping path in its
Rust unit tests.  This script reads those test modules as text (it runs nothing) and
writes the inputs and expected outputs as JSON fixtures for tests/test_unit_vectors.py:

* src/piecewisealigner.rs: global_alignment, xdrop_alignment (both modes),
  remove_spurious_anchors and extend_piecewise cases (score, spans, CIGAR, edit distance)
* src/aligner.rs: highest_scoring_segment, hamming_align, hamming_align_global, and the
  Aligner::align None / Some cases
* src/chainer.rs: collinear_chaining best-score properties
* src/mapper.rs: has_shared_substring cases
* src/seeding/hash.rs: the xxh64 known answer; src/indexer.rs: pick_bits on phiX

Usage: extract_unit_vectors.py REFERENCE_TREE   (or STROBEALIGN_REFERENCE=... in the
environment); the tree is the strobealign source checkout.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

OUT = Path(__file__).resolve().parent / "unit_vectors.json"


def tests_of(text: str) -> list[tuple[str, str]]:
    """(name, body) of every #[test] function."""
    out = []
    for m in re.finditer(r"#\[test\]\s*(?:#\[[^\]]*\]\s*)*fn (\w+)\(\)\s*\{", text):
        i, depth = m.end(), 1
        while depth:
            c = text[i]
            depth += c == "{"
            depth -= c == "}"
            i += 1
        out.append((m.group(1), text[m.end():i - 1]))
    return out


def arith(expr: str) -> int:
    expr = expr.strip().rstrip(",")
    if not re.fullmatch(r"[0-9+\-*() ]+", expr):
        raise ValueError(f"not an integer expression: {expr!r}")
    return int(eval(expr, {"__builtins__": {}}, {}))  # digits and + - * ( ) only


def bstrings(s: str) -> list[str]:
    return re.findall(r'b"([^"]*)"', s)


def vec_after(body: str, var: str) -> list[dict]:
    m = re.search(r"let (?:mut )?" + var + r"\s*=\s*vec!\[", body)
    if not m:
        return []
    i, depth = m.end(), 1
    while depth:
        depth += body[i] == "["
        depth -= body[i] == "]"
        i += 1
    seg = body[m.end():i - 1]
    return [dict(ref_id=int(a), ref_start=int(b), query_start=int(c)) for a, b, c in re.findall(
        r"Anchor\s*\{\s*ref_id:\s*(\d+),\s*ref_start:\s*(\d+),\s*query_start:\s*(\d+),?\s*\}", seg)]


def asserts(body: str, obj: str) -> dict:
    """assert_eq!(obj.field, expr) and assert_eq!(obj.cigar.to_string(), "...")."""
    exp = {}
    for f, e in re.findall(r"assert_eq!\(\s*" + obj + r"\.(\w+)(?:\(\))?\s*,\s*([^;]*?)\s*,?\s*\);", body):
        if f == "cigar":
            continue
        exp[f] = arith(e)
    m = re.search(r"assert_eq!\(\s*" + obj + r'\.cigar\.to_string\(\)\s*,\s*"([^"]*)"\s*\)', body)
    if m:
        exp["cigar"] = m.group(1)
    if re.search(r"assert!\(\s*" + obj + r"\.cigar\.is_empty\(\)\s*\)", body):
        exp["cigar"] = ""
    return exp


def scores(body: str) -> dict:
    m = re.search(r"Scores\s*\{([^}]*)\}", body)
    kv = dict(re.findall(r"(\w+):\s*(\d+)", m.group(1)))
    return {"match": int(kv["match_"]), "mismatch": int(kv["mismatch"]), "gap_open": int(kv["gap_open"]),
            "gap_extend": int(kv["gap_extend"]), "end_bonus": int(kv["end_bonus"])}


def piecewise(text: str) -> list[dict]:
    cases = []
    for name, body in tests_of(text):
        c: dict = {"name": name}
        if "remove_spurious_anchors(" in body:
            c["kind"] = "remove_spurious_anchors"
            exp = vec_after(body, "expected")
            inp = vec_after(body, "result")
            c["anchors"] = inp or exp
            c["expected"] = exp
            cases.append(c)
            continue
        c["scores"] = scores(body)
        m = re.search(r"PiecewiseAligner::new\(\s*Scores\s*\{[^}]*\}\s*,\s*(\d+)\s*,\s*(\d+)", body)
        c["k"], c["xdrop"] = int(m.group(1)), int(m.group(2))
        if "global_alignment(" in body:
            c["kind"] = "global"
            c["query"], c["ref"] = bstrings(body[body.index("global_alignment("):])[:2]
        elif "xdrop_alignment(" in body:
            c["kind"] = "xdrop_" + re.search(r"XdropMode::(\w+)", body).group(1)
            c["query"], c["ref"] = bstrings(body[body.index("xdrop_alignment("):])[:2]
        elif "extend_piecewise(" in body:
            c["kind"] = "extend_piecewise"
            c["query"] = re.search(r'let query\s*=\s*b"([^"]*)"', body).group(1)
            c["ref"] = re.search(r'let refseq\s*=\s*b"([^"]*)"', body).group(1)
            c["anchors"] = vec_after(body, "anchors")
            c["padding"] = int(re.search(r"extend_piecewise\([^)]*,\s*(\d+)\s*\)", body).group(1))
        else:
            continue
        if re.search(r"assert!\(\s*result\.is_none\(\)\s*\)", body):
            c["expected"] = None
        else:
            c["expected"] = asserts(body, "result")
        cases.append(c)
    return cases


def aligner(text: str) -> dict:
    hss, ham, glob, align = [], [], [], []
    for name, body in tests_of(text):
        if "highest_scoring_segment(" in body:
            for q, r, a, b, e, exp in re.findall(
                    r'assert_eq!\(\s*highest_scoring_segment\(b"([^"]*)",\s*b"([^"]*)",\s*(\d+),\s*(\d+),\s*(\d+)\),'
                    r"\s*\(([^;]*)\)\s*\);", body):
                s, t, sc = [x for x in re.split(r",(?![^()]*\))", exp) if x.strip()]
                hss.append({"name": name, "query": q, "ref": r, "match": int(a), "mismatch": int(b),
                            "end_bonus": int(e), "expected": [arith(s), arith(t), arith(sc)]})
            for m in re.finditer(r'let \(start, end, _score\) = highest_scoring_segment\(b"([^"]*)",\s*b"([^"]*)",'
                                 r"\s*(\d+),\s*(\d+),\s*(\d+)\);\s*assert_eq!\(start, (\d+)\);\s*assert_eq!\(end, "
                                 r"(\d+)\);", body):
                q, r, a, b, e, s, t = m.groups()
                hss.append({"name": name, "query": q, "ref": r, "match": int(a), "mismatch": int(b),
                            "end_bonus": int(e), "expected": [int(s), int(t), None]})
        elif "hamming_align(" in body:
            q, r = bstrings(body)[:2]
            a, b, e = map(int, re.search(r'hamming_align\(b"[^"]*",\s*b"[^"]*",\s*(\d+),\s*(\d+),\s*(\d+)\)',
                                         body).groups())
            ham.append({"name": name, "query": q, "ref": r, "match": a, "mismatch": b, "end_bonus": e,
                        "expected": asserts(body, "info")})
        elif "hamming_align_global(" in body:
            q, r = bstrings(body)[:2]
            a, b = map(int, re.search(r'hamming_align_global\(b"[^"]*",\s*b"[^"]*",\s*(\d+),\s*(\d+)\)',
                                      body).groups())
            glob.append({"name": name, "query": q, "ref": r, "match": a, "mismatch": b,
                         "expected": asserts(body, "info")})
        elif "aligner.align(" in body:
            q = re.search(r'let query\s*=\s*b"([^"]*)"', body).group(1)
            r = re.search(r'let refseq\s*=\s*b"([^"]*)"', body).group(1)
            some = "is_some()" in body
            align.append({"name": name, "query": q, "ref": r, "some": some})
    return {"highest_scoring_segment": hss, "hamming_align": ham, "hamming_align_global": glob, "align": align}


def chainer(text: str) -> list[dict]:
    out = []
    for name, body in tests_of(text):
        k = int(re.search(r"Chainer::new\((\d+)", body).group(1))
        anchors = vec_after(body, "anchors")
        if not anchors:
            seg = body[body.index("let anchors"):]
            anchors = [dict(ref_id=int(a), ref_start=int(b), query_start=int(c)) for a, b, c in re.findall(
                r"Anchor\s*\{\s*ref_id:\s*(\d+),\s*ref_start:\s*(\d+),\s*query_start:\s*(\d+),?\s*\}", seg)]
        gaps = [int(x) for x in re.findall(r"collinear_chaining\([^,]*,\s*(\d+)\)", body)]
        c = {"name": name, "k": k, "anchors": anchors, "max_ref_gap": gaps[0]}
        m = re.search(r"assert!\(chaining_result\.best_score > ([0-9.]+)\)", body)
        if m:
            c["best_score_above"] = float(m.group(1))
        if "chainer.k as f32" in body:
            c["best_score_equals_k"] = True
        if "score1 * 2.0" in body:
            c["linear_prefixes"] = [1, 2, 3]
        out.append(c)
    return out


def shared_substring(text: str) -> list[dict]:
    out = []
    for name, body in tests_of(text):
        m = re.search(r"(!?)has_shared_substring\(\s*(?:b\"([^\"]*)\"|\"([^\"]*)\"\.as_bytes\(\)),\s*"
                      r"(?:b\"([^\"]*)\"|\"([^\"]*)\"\.as_bytes\(\)),\s*(\d+)\s*\)", body)
        if m:
            neg, a1, a2, b1, b2, k = m.groups()
            out.append({"name": name, "read": a1 if a1 is not None else a2, "ref": b1 if b1 is not None else b2,
                        "k": int(k), "expected": not neg})
    return out


def main() -> None:
    tree = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STROBEALIGN_REFERENCE", ""))
    if not str(tree) or not (tree / "src" / "piecewisealigner.rs").exists():
        sys.exit("usage: extract_unit_vectors.py REFERENCE_TREE (the strobealign source checkout)")
    src = tree / "src"
    hash_rs = (src / "seeding" / "hash.rs").read_text()
    m = re.search(r"assert_eq!\(xxh64\((0x[0-9a-fA-F]+)u64\),\s*(0x[0-9a-fA-F]+)\)", hash_rs)
    idx_rs = (src / "indexer.rs").read_text()
    pb = re.search(r"fn pick_bits\(\)\s*\{(.*?)\n    \}", idx_rs, re.S).group(1)
    k, s = map(int, re.search(r"SyncmerParameters::try_new\((\d+),\s*(\d+)\)", pb).groups())
    bits = int(re.search(r"pick_bits\(&references\),\s*(\d+)\)", pb).group(1))
    data = {
        "source": "strobealign unit tests (src/piecewisealigner.rs, src/aligner.rs, src/chainer.rs, src/mapper.rs, "
                  "src/seeding/hash.rs, src/indexer.rs), extracted by tests/golden/extract_unit_vectors.py",
        "xxh64": [{"input": m.group(1), "expected": m.group(2)}],
        "pick_bits": [{"fasta": "phix.fasta", "k": k, "s": s, "expected": bits}],
        "piecewise": piecewise((src / "piecewisealigner.rs").read_text()),
        "chaining": chainer((src / "chainer.rs").read_text()),
        "has_shared_substring": shared_substring((src / "mapper.rs").read_text()),
    }
    data.update(aligner((src / "aligner.rs").read_text()))
    OUT.write_text(json.dumps(data, indent=1) + "\n")
    counts = {k: len(v) for k, v in data.items() if isinstance(v, list)}
    print(f"wrote {OUT}: {counts}")


if __name__ == "__main__":
    main()
