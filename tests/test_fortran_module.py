"""The Fortran iso_c_binding module (include/derek_gpu.f90) against the C
header it binds, checked statically (no Fortran compiler is needed):

* every function of include/derek_gpu.h has exactly one interface, and the
  library exports each bound name;
* argument counts agree, and each argument's kind and passing agree with its
  C declaration: a C scalar is a Fortran `value` of the matching kind, a C
  pointer or array is a by-reference dummy of the pointee's kind or a
  `type(c_ptr), value`;
* the bind(C) derived types list the C structs' members in order, with the
  same kinds and array lengths;
* the status, precision and grid-policy constants carry the header's values;
* the Python package's ctypes signatures agree with the same prototypes.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "derek_gpu.h")
MODULE = os.path.join(ROOT, "include", "derek_gpu.f90")

C_KIND = {"int": "c_int", "long": "c_long", "long long": "c_long_long", "double": "c_double",
          "int32_t": "c_int32_t", "uint64_t": "c_int64_t", "char": "c_char", "void": "c_ptr",
          "unsigned long long": "c_long_long"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", " ", s, flags=re.S)


def c_header():
    src = _strip_c_comments(open(HEADER).read())
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(DEREK_\w+)\s+(-?\d+)", src)}
    body = re.sub(r"#.*", " ", src)
    structs = {}
    for m in re.finditer(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", body, flags=re.S):
        members = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            base = re.match(r"(const\s+)?(unsigned long long|long long|\w+)\s*(\*?)\s*(.*)", decl)
            ctype, ptr, names = base.group(2), base.group(3), base.group(4)
            for nm in names.split(","):
                nm = nm.strip()
                star = ptr or nm.startswith("*")
                nm = nm.lstrip("*").strip()
                am = re.match(r"(\w+)\s*(?:\[(.*?)\])?", nm)
                length = 1 if am.group(2) is None else eval(am.group(2))
                members.append((am.group(1), "c_ptr" if star else C_KIND[ctype], length))
        structs[m.group(2)] = members
    funcs = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(derek_\w+)\s*\(([^;{]*?)\)\s*;", body, flags=re.S):
        name, args = m.group(2), " ".join(m.group(3).split())
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        funcs[name] = params
    return consts, structs, funcs


def f90_module():
    text = open(MODULE).read()
    lines = []
    for raw in text.split("\n"):
        raw = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + raw.strip().lstrip("&")
        else:
            lines.append(raw)
    consts = {}
    for ln in lines:
        m = re.match(r"\s*integer\(c_int\),\s*parameter\s*::\s*(.*)", ln)
        if m:
            for item in m.group(1).split(","):
                k, v = item.split("=")
                consts[k.strip()] = int(v)
    types, cur = {}, None
    for ln in lines:
        m = re.match(r"\s*type,\s*bind\(C\)\s*::\s*(\w+)", ln)
        if m:
            cur = m.group(1)
            types[cur] = []
            continue
        if cur and re.match(r"\s*end type", ln):
            cur = None
            continue
        if cur:
            m = re.match(r"\s*(integer|real|character|type)\((?:kind=)?(\w+)\)\s*::\s*(.*)", ln)
            for nm in re.finditer(r"(\w+)(?:\((\d+)\))?", m.group(3)):
                types[cur].append((nm.group(1), m.group(2), int(nm.group(2) or 1)))
    ifaces, cur = {}, None
    for ln in lines:
        m = re.match(r"\s*(?:([\w\(\)]+)\s+)?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", ln)
        if m:
            assert m.group(3) == m.group(5), f"interface {m.group(3)} binds {m.group(5)}"
            cur = {"args": [a.strip() for a in m.group(4).split(",") if a.strip()], "decl": {}}
            ifaces[m.group(5)] = cur
            continue
        if cur is not None and re.match(r"\s*end (function|subroutine)", ln):
            cur = None
            continue
        if cur is not None:
            m = re.match(r"\s*(integer|real|complex|character|type)\((?:kind=)?(\w+)\)\s*(,[^:]*)?::\s*(.*)", ln)
            if m:
                attrs = m.group(3) or ""
                for nm in re.finditer(r"(\w+)(?:\(([^)]*)\))?", m.group(4)):
                    cur["decl"][nm.group(1)] = (m.group(1), m.group(2), "value" in attrs, nm.group(2))
    return consts, types, ifaces


def _c_param(p):
    """(kind, is_pointer) of one C parameter declaration."""
    p = p.replace("const ", "").strip()
    m = re.match(r"(unsigned long long|long long|\w+)\s*(\*\*|\*)?\s*(\w+)?\s*(\[\w*\])?", p)
    ctype, star, arr = m.group(1), m.group(2), m.group(4)
    if ctype.startswith("derek_") and ctype != "derek_gpu_t":
        return ctype, True
    if ctype == "derek_gpu_t":
        return ("c_ptr", star == "**") if star else ("c_ptr", False)
    return C_KIND[ctype], bool(star or arr)


def test_constants_match():
    c, _, _ = c_header()
    f, _, _ = f90_module()
    for name, val in f.items():
        assert c[name] == val, name
    for name in ("DEREK_OK", "DEREK_ERR_UNSUPPORTED", "DEREK_PREC_MIXED", "DEREK_GRID_SMOOTH23"):
        assert name in f


def test_derived_types_match_structs():
    _, structs, _ = c_header()
    _, types, _ = f90_module()
    for name in ("derek_sys_desc", "derek_scf_opts", "derek_scf_report", "derek_info"):
        cm, fm = structs[name], types[name]
        assert [m[0] for m in cm] == [m[0] for m in fm], name
        for (n, ck, cl), (_, fk, fl) in zip(cm, fm):
            assert ck == fk and cl == fl, (name, n, ck, fk, cl, fl)


def test_every_function_bound_with_matching_arguments():
    _, _, funcs = c_header()
    _, _, ifaces = f90_module()
    assert sorted(funcs) == sorted(ifaces), set(funcs) ^ set(ifaces)
    for name, params in funcs.items():
        f = ifaces[name]
        assert len(params) == len(f["args"]), name
        for p, arg in zip(params, f["args"]):
            kind, is_ptr = _c_param(p)
            fkind, ftyp, value, dims = f["decl"][arg][1], f["decl"][arg][0], f["decl"][arg][2], f["decl"][arg][3]
            if kind == "c_ptr" and not is_ptr:                       # the handle, void *, by value
                assert ftyp == "type" and fkind == "c_ptr" and value, (name, arg)
            elif not is_ptr:                                          # C scalar: by value
                assert value and fkind == kind, (name, arg, kind, fkind)
            elif ftyp == "type" and fkind == "c_ptr" and value:      # a NULL-able pointer
                pass
            else:                                                     # by reference
                assert not value, (name, arg)
                want = {kind} | ({"c_double_complex"} if kind == "c_double" else set())
                if kind.startswith("derek_"):
                    want = {kind}
                if kind == "c_ptr":                                   # derek_gpu_t **
                    want = {"c_ptr"}
                assert fkind in want, (name, arg, kind, fkind)


def test_bound_names_exported():
    import derek_gb300 as dg
    _, _, ifaces = f90_module()
    for name in ifaces:
        assert hasattr(dg.lib, name), name


def _ctypes_kind(t):
    """(kind, is_pointer) of a ctypes argument type."""
    import ctypes
    if t in (ctypes.c_void_p, ctypes.c_char_p):
        return ("c_ptr" if t is ctypes.c_void_p else "c_char"), True
    scalars = {ctypes.c_int: "c_int", ctypes.c_long: "c_long", ctypes.c_longlong: "c_long_long",
               ctypes.c_double: "c_double", ctypes.c_uint64: "c_int64_t"}
    if t in scalars:
        return scalars[t], False
    target = getattr(t, "_type_", None)
    if target is not None and not isinstance(target, str):
        if target in scalars:
            return scalars[target], True
        return "struct", True
    raise AssertionError(f"unmapped ctypes type {t}")


def test_ctypes_signatures_match_header():
    """derek_gb300's ctypes argument lists against the C prototypes: every
    declared function has a signature with the same count of arguments, and
    each scalar / pointer agrees with its C declaration."""
    from derek_gb300 import _abi
    _, _, funcs = c_header()
    missing = sorted(set(funcs) - set(_abi.SIGNATURES))
    assert not missing, missing
    for name, (_, args) in _abi.SIGNATURES.items():
        params = funcs[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for t, p in zip(args, params):
            kind, is_ptr = _c_param(p)
            ckind, cptr = _ctypes_kind(t)
            if kind == "c_ptr" and not is_ptr:          # handle or void * by value
                assert ckind == "c_ptr", (name, p)
                continue
            assert cptr == is_ptr, (name, p, t)
            if not is_ptr:
                # LP64 (x86_64 and aarch64 Linux): ctypes.c_long is c_longlong, both 8 bytes
                same = {kind, ckind} <= {"c_long", "c_long_long"}
                assert ckind == kind or same, (name, p, t)
            elif ckind not in ("c_ptr", "struct", "c_char"):
                assert ckind == kind or (kind == "c_int32_t" and ckind == "c_int"), (name, p, t)
