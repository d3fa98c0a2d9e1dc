"""Extract the reference's own known answers into tests/golden/reference_benchmarks.json.

Run in a container where the reference checkout is present:

    python tests/golden/make_reference_goldens.py /path/to/TeaLeaf_ref

It reads, from the reference's files only:
  * Benchmarks/tea_bm_{1..6}.in  -- the input decks (verbatim text),
  * Benchmarks/tea_bm_{1..6}.out -- field summaries (step, volume, mass, density,
    internal energy, temperature) and the per-step "Conduction error" /
    "Iteration count" lines,
  * tea.in                       -- the PPCG deck (halo_depth 2, test problem 4),
  * field_summary.f90            -- the QA constants for test problems 1..6.
The JSON it writes is committed, so the tests never need the reference checkout.
"""
import json
import os
import re
import sys


def parse_out(text):
    summaries = []
    for m in re.finditer(r"^\s*step:\s+(\d+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s*$", text, re.M):
        step = int(m.group(1))
        vals = [float(m.group(i)) for i in range(2, 7)]
        summaries.append({"step": step, "volume": vals[0], "mass": vals[1], "density": vals[2],
                          "energy": vals[3], "temperature": vals[4]})
    # keep the first occurrence per step (the final summary is printed twice)
    seen, uniq = set(), []
    for s in summaries:
        if s["step"] not in seen:
            seen.add(s["step"])
            uniq.append(s)
    iters = [int(x) for x in re.findall(r"^\s*Iteration count\s+(\d+)", text, re.M)]
    errs = [float(x) for x in re.findall(r"^\s*Conduction error\s+(\S+)", text, re.M)]
    tasks = re.search(r"Task Count\s+(\d+)", text)
    version = re.search(r"Tea Version\s+(\S+)", text)
    return {"summaries": uniq, "iterations": iters, "conduction_errors": errs,
            "task_count": int(tasks.group(1)) if tasks else None,
            "version": version.group(1) if version else None}


def main(ref):
    out = {"source": "UK-MAC/TeaLeaf_ref Benchmarks/*.out, tea.in, field_summary.f90", "benchmarks": {}}
    for i in range(1, 7):
        deck = open(os.path.join(ref, "Benchmarks", "tea_bm_%d.in" % i)).read()
        res = parse_out(open(os.path.join(ref, "Benchmarks", "tea_bm_%d.out" % i)).read())
        res["deck"] = deck
        out["benchmarks"]["tea_bm_%d" % i] = res
    out["ppcg_deck"] = open(os.path.join(ref, "tea.in")).read()
    fs = open(os.path.join(ref, "field_summary.f90")).read()
    qa = {}
    for m in re.finditer(r"test_problem\.EQ\.(\d+)\)\s*qa_diff=ABS\(\(100\.0_8\*\(temp/([0-9.]+)_8\)\)", fs):
        qa[m.group(1)] = float(m.group(2))
    out["qa_temperature"] = qa
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_benchmarks.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_goldens.py <path to the TeaLeaf_ref source tree>")
    main(sys.argv[1])
