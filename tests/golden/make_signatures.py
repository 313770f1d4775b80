"""Extract the positional signatures of the reference functions that the Julia
binding (merzbild.jl_gb300/julia/MerzbildGPU.jl) mirrors, into
tests/golden/reference_signatures.json (committed).

Usage: python tests/golden/make_signatures.py <reference checkout>/src

Every `function name(args; kwargs)` definition of the listed names in the
source tree is recorded with its file, line and positional argument names
(type annotations and default values stripped)."""
import json
import os
import re
import sys

NAMES = ["ntc!", "ntc_equal_weight!", "compute_props!", "compute_props_sorted!", "compute_props_with_total_moments!",
         "convect_particles!", "sort_particles!", "merge_octree_N2_based!", "squash_pia!",
         "create_collision_factors_array", "check_pia_is_correct", "check_unique_index", "check_unique_buffer",
         "count_disordered_particles"]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_signatures.json")


def split_args(text):
    """Top-level comma split (no splitting inside brackets or braces)."""
    out, depth, cur = [], 0, ""
    for ch in text:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [a.strip() for a in out]


def arg_name(a):
    a = a.split("=")[0]
    return a.split("::")[0].strip()


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_signatures.py <reference src directory>")
    src = sys.argv[1]
    found = []
    pat = re.compile(r"^(?:@inline\s+)?function\s+([A-Za-z_][A-Za-z0-9_!]*)\s*\(")
    for root, _, files in os.walk(src):
        for fn in sorted(files):
            if not fn.endswith(".jl"):
                continue
            path = os.path.join(root, fn)
            lines = open(path, encoding="utf-8").read().splitlines()
            for i, ln in enumerate(lines):
                m = pat.match(ln)
                if not m or m.group(1) not in NAMES:
                    continue
                # the argument list may continue over several lines
                text = ln[m.end():]
                k = i
                depth = 1
                buf = ""
                while True:
                    for ch in text:
                        if ch == "(":
                            depth += 1
                        elif ch == ")":
                            depth -= 1
                            if depth == 0:
                                break
                        buf += ch
                    if depth == 0:
                        break
                    k += 1
                    text = lines[k]
                    buf += " "
                pos = buf.split(";")[0]
                args = [arg_name(a) for a in split_args(pos)]
                found.append({"name": m.group(1), "file": os.path.relpath(path, os.path.dirname(src)),
                              "line": i + 1, "args": args})
    found.sort(key=lambda r: (r["name"], r["file"], r["line"]))
    with open(OUT, "w") as f:
        json.dump(found, f, indent=1, ensure_ascii=False)
    print(f"wrote {len(found)} signatures to {OUT}")


if __name__ == "__main__":
    main()
