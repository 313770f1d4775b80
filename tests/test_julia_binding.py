"""CPU checks of the Julia binding (merzbild.jl_gb300/julia/MerzbildGPU.jl),
which cannot run here (no Julia toolchain):

* the drop-in methods: every reference function of the path that takes
  particles, a ParticleIndexerArray or collision factors has a method of the
  same name on the device containers with the same positional arguments, in
  the same order (the reference's signatures are the committed fixture
  tests/golden/reference_signatures.json, extracted from its source by
  tests/golden/make_signatures.py);
* every ccall passes the argument types of the entry point's prototype in
  include/merzgpu.h, in number and kind."""
import json
import os
import re

import pytest

from conftest import ROOT

JL = os.path.join(ROOT, "merzbild.jl_gb300", "julia", "MerzbildGPU.jl")
HEADER = os.path.join(ROOT, "include", "merzgpu.h")


def _split_top(text, sep=","):
    out, depth, cur = [], 0, ""
    for ch in text:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [a.strip() for a in out]


def _balanced(text, start):
    """Contents of the parenthesis opened at text[start]."""
    depth = 0
    for k in range(start, len(text)):
        if text[k] == "(":
            depth += 1
        elif text[k] == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:k]
    raise ValueError("unbalanced")


def shim_methods():
    """(name, positional argument names) of every method the binding adds to
    Merzbild's functions."""
    src = open(JL, encoding="utf-8").read()
    out = []
    for m in re.finditer(r"(?m)^(?:function\s+)?Merzbild\.([A-Za-z_][A-Za-z0-9_!]*)\(", src):
        args = _balanced(src, m.end() - 1)
        pos = _split_top(args.split(";")[0])
        out.append((m.group(1), [a.split("=")[0].split("::")[0].strip() for a in pos]))
    return out


def test_drop_in_methods_keep_the_reference_signatures():
    with open(os.path.join(ROOT, "tests", "golden", "reference_signatures.json"), encoding="utf-8") as f:
        ref = json.load(f)
    methods = shim_methods()
    assert len(methods) >= 20
    # host-only constructors of the reference (species and cell counts) have no device form
    host_only = {("create_collision_factors_array", ("n_species",)),
                 ("create_collision_factors_array", ("n_species", "n_cells"))}
    missing = []
    for r in ref:
        key = (r["name"], tuple(r["args"]))
        if key in host_only:
            continue
        if (r["name"], r["args"]) not in [(n, a) for n, a in methods]:
            missing.append(f'{r["name"]}({", ".join(r["args"])})  {r["file"]}:{r["line"]}')
    assert not missing, "no device method with the reference's positional arguments:\n" + "\n".join(missing)
    # and no device method that the reference does not have
    names = {r["name"] for r in ref}
    extra = [(n, a) for n, a in methods if n in names and (n, a) not in [(r["name"], r["args"]) for r in ref]]
    assert not extra, extra


# ------------------------------------------------------------------ ccall argument types
_PTR = re.compile(r"^(?:Ptr|Ref)\{(.+)\}$")


def c_kind(ctype):
    """Kind of a C parameter type: ('scalar', name) or ('ptr', pointee kind)."""
    t = ctype.replace("const", "").strip()
    t = re.sub(r"\s+", " ", t)
    if t.endswith("*"):
        inner = t[:-1].strip()
        return ("ptr", c_kind(inner) if inner.endswith("*") else inner)
    return ("scalar", t)


def jl_kind(jtype):
    t = jtype.strip()
    if t == "Cstring":  # Julia's NUL-terminated char*
        return ("ptr", "char")
    m = _PTR.match(t)
    if m:
        inner = m.group(1).strip()
        return ("ptr", jl_kind(inner) if (_PTR.match(inner) or inner == "Cstring") else inner)
    return ("scalar", t)


SCALARS = {
    "int32_t": {"Int32", "Cint"}, "int": {"Cint", "Int32"}, "int64_t": {"Int64"}, "uint64_t": {"UInt64"},
    "double": {"Float64"}, "size_t": {"Csize_t", "UInt64"}, "uint32_t": {"UInt32"},
}
POINTEES = {
    "void": {"Cvoid"}, "mz_ctx": {"Cvoid"}, "mz_domain": {"Cvoid"}, "mz_props": {"Cvoid"}, "mz_surf_props": {"Cvoid"},
    "mz_server": {"Cvoid"}, "mz_nc_file": {"Cvoid"}, "char": {"char", "UInt8", "Cchar", "Cvoid"}, "double": {"Float64"},
    "int32_t": {"Int32"}, "int64_t": {"Int64"}, "uint64_t": {"UInt64"}, "uint32_t": {"UInt32"},
    "mz_grid1d": {"DeviceGrid1D"}, "mz_walls1d": {"DeviceWalls1D"}, "mz_octree_params": {"DeviceOctree"},
    "mz_step_plan": {"MzStepPlan"}, "mz_interaction": {"MzInteraction"}, "mz_particle_indexer": {"MzParticleIndexer"},
    "mz_collision_factors": {"MzCollisionFactors"}, "mz_counters": {"MzCounters"}, "mz_request": {"MzRequest"},
    "mz_request_result": {"MzRequestResult"}, "mz_nc_attribute": {"MzNcAttribute"},
}


def compatible(ck, jk):
    if ck[0] != jk[0]:
        return False
    if ck[0] == "scalar":
        return jk[1] in SCALARS.get(ck[1], {ck[1]})
    if isinstance(ck[1], tuple) or isinstance(jk[1], tuple):
        # pointer to pointer (an out handle): Ref{Ptr{Cvoid}}
        return isinstance(ck[1], tuple) and isinstance(jk[1], tuple)
    return jk[1] in POINTEES.get(ck[1], {ck[1]}) or jk[1] == "Cvoid"


def header_prototypes():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    protos = {}
    for m in re.finditer(r"\bint\s+(mz_\w+)\s*\(([^)]*)\)\s*;", txt):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        kinds = []
        for p in params:
            p = re.sub(r"\[[^\]]*\]", "*", p)  # array parameters are pointers
            name = re.match(r"(.*?)(\w+)\s*$", p)
            kinds.append(c_kind(name.group(1)))
        protos[m.group(1)] = kinds
    return protos


def shim_ccalls():
    src = open(JL, encoding="utf-8").read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(mz_\w+),\s*libmz\)\s*,", src):
        body = _balanced(src, m.start() + len("ccall"))
        parts = _split_top(body)
        types = parts[2]
        assert types.startswith("(") and types.endswith(")"), (m.group(1), types)
        tlist = _split_top(types[1:-1])
        calls.append((m.group(1), [jl_kind(t) for t in tlist], parts[1].strip()))
    return calls


def test_ccall_argument_types_match_the_header():
    protos = header_prototypes()
    calls = shim_ccalls()
    assert len(calls) > 40
    bad = []
    for name, jks, ret in calls:
        assert ret == "Cint", (name, ret)
        cks = protos[name]
        if len(cks) != len(jks):
            bad.append(f"{name}: {len(jks)} arguments, the header declares {len(cks)}")
            continue
        for i, (ck, jk) in enumerate(zip(cks, jks)):
            if not compatible(ck, jk):
                bad.append(f"{name} argument {i + 1}: C {ck} vs Julia {jk}")
    assert not bad, "\n".join(bad)


def test_julia_structs_match_the_header_layouts():
    """Field counts and kinds of the structs the binding passes by reference."""
    src = open(JL, encoding="utf-8").read()
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)

    def c_body(name):
        end = re.search(r"\}\s*" + name + r"\s*;", txt)
        start = txt.rfind("typedef struct", 0, end.start())
        return txt[txt.index("{", start) + 1:end.start()]

    def c_fields(name):
        body = c_body(name)
        n = 0
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            typ, rest = decl.split(None, 1) if not decl.startswith("unsigned long long") else (
                "unsigned long long", decl[len("unsigned long long"):])
            for v in rest.split(","):
                dims = [int(x) if x.isdigit() else 4 for x in re.findall(r"\[(\w+)\]", v)]
                k = 1
                for x in dims:
                    k *= x
                n += k
        return n

    def jl_fields(name):
        m = re.search(r"struct " + name + r"\b(.*?)\nend", src, flags=re.S)
        body = re.sub(r"#.*", "", m.group(1))
        n = 0
        for decl in re.split(r"[;\n]", body):
            decl = decl.strip()
            if "::" not in decl:
                continue
            typ = decl.split("::", 1)[1].strip()
            t = re.match(r"NTuple\{(\d+|[A-Z_ *0-9]+),", typ)
            if t:
                expr = t.group(1).replace("MZ_MAX_SPECIES", "4")
                n += eval(expr)
            else:
                n += 1
        return n

    # (C struct, Julia struct): scalar slots
    for c_name, j_name in (("mz_grid1d", "DeviceGrid1D"), ("mz_walls1d", "DeviceWalls1D"),
                           ("mz_octree_params", "DeviceOctree"), ("mz_particle_indexer", "MzParticleIndexer")):
        assert c_fields(c_name) == jl_fields(j_name), (c_name, c_fields(c_name), jl_fields(j_name))
    # the step plan: same field order, nested structs by name
    body = c_body("mz_step_plan")
    c_names = [n for d in body.split(";") if d.strip() for n in [x.strip().split()[-1] for x in d.strip().split(",")]]
    mj = re.search(r"struct MzStepPlan\b(.*?)\nend", src, flags=re.S)
    j_names = [d.split("::")[0].strip() for d in re.split(r"[;\n]", re.sub(r"#.*", "", mj.group(1))) if "::" in d]
    assert c_names == j_names, (c_names, j_names)
