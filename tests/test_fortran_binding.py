"""The Fortran module include/ns_gpu.f90 against the C header include/ns_gpu.h.

No Fortran compiler exists on either machine, so the binding is checked as
text: every function the header declares has a bind(C) interface of the
same name and the same number of arguments, each argument passed by value
exactly where the header passes a scalar by value, and every
``type, bind(C)`` lists its C struct's fields in the same order with the
interoperable kind (int -> c_int, double -> c_double, long long ->
c_long_long, char -> c_char) and the same array extents.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ns_gpu.h")
F90 = os.path.join(ROOT, "include", "ns_gpu.f90")

C2F = {"int": "c_int", "double": "c_double", "long long": "c_long_long", "char": "c_char"}


def _c_source():
    return re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)


def c_prototypes():
    """{name: [(is_pointer_or_array, text), ...]} of every ns_* function."""
    src = _c_source()
    out = {}
    for m in re.finditer(r"(?:^|\n)\s*(?:const\s+)?[A-Za-z_][\w ]*?\**\s*(ns_\w+)\s*\(([^()]*)\)\s*;", src):
        args = [a.strip() for a in m.group(2).split(",")]
        if args == ["void"] or args == [""]:
            args = []
        out[m.group(1)] = [("*" in a or "[" in a, a) for a in args]
    return out


def c_structs():
    """{typedef name: [(field, c type, extent), ...]}."""
    src = _c_source()
    out = {}
    for m in re.finditer(r"typedef\s+struct\s+\w+\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mm = re.match(r"(long long|int|double|char)\s+(.*)", decl)
            assert mm, decl
            for item in mm.group(2).split(","):
                item = item.strip()
                a = re.match(r"(\w+)(?:\[(\d+)\])?$", item)
                fields.append((a.group(1), mm.group(1), int(a.group(2) or 1)))
        out[m.group(2)] = fields
    return out


def _f90_lines():
    lines, buf = [], ""
    for raw in open(F90):
        line = raw.split("!")[0].rstrip()
        if buf:
            line = buf + " " + line.lstrip().lstrip("&")
            buf = ""
        if line.endswith("&"):
            buf = line[:-1]
            continue
        lines.append(line)
    return lines


def f90_interfaces():
    """{bind name: (dummy names, {dummy: declaration line})}."""
    lines = _f90_lines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.search(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", lines[i])
        if m:
            dummies = [d.strip().lower() for d in m.group(2).split(",") if d.strip()]
            decls = {}
            i += 1
            while not re.match(r"\s*end\s+(function|subroutine)", lines[i]):
                dm = re.match(r"\s*(.*?)::(.*)", lines[i])
                if dm:
                    for name in re.findall(r"(\w+)(?:\([^)]*\))?", dm.group(2)):
                        decls[name.lower()] = dm.group(1).lower()
                i += 1
            out[m.group(3)] = (dummies, decls)
        i += 1
    return out


def f90_types():
    """{type name: [(field, kind, extent), ...]} of every type, bind(C)."""
    lines = _f90_lines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"\s*type,\s*bind\(C\)\s*::\s*(\w+)", lines[i])
        if m:
            fields = []
            i += 1
            while not re.match(r"\s*end\s+type", lines[i]):
                dm = re.match(r"\s*(integer|real|character)\((?:kind=)?(\w+)\)\s*::(.*)", lines[i])
                if dm:
                    for name, ext in re.findall(r"(\w+)(?:\((\d+)\))?", dm.group(3)):
                        fields.append((name, dm.group(2), int(ext or 1)))
                i += 1
            out[m.group(1)] = fields
        i += 1
    return out


def test_every_header_function_has_a_fortran_interface():
    c = c_prototypes()
    f = f90_interfaces()
    assert len(c) > 60
    missing = sorted(set(c) - set(f))
    assert not missing, missing


def test_argument_counts_and_value_passing_agree():
    c = c_prototypes()
    f = f90_interfaces()
    for name, args in c.items():
        dummies, decls = f[name]
        assert len(dummies) == len(args), (name, dummies, args)
        for (is_ptr, text), d in zip(args, dummies):
            decl = decls.get(d)
            assert decl is not None, (name, d)
            by_value = "value" in decl
            if is_ptr:
                # a C pointer is a Fortran reference, or a c_ptr passed by value
                assert not by_value or "type(c_ptr)" in decl, (name, d, text, decl)
            else:
                assert by_value, (name, d, text, decl)


def test_bind_c_types_match_the_c_structs_field_by_field():
    cs = c_structs()
    ft = f90_types()
    for cname, fname in (("ns_config", "ns_config"), ("ns_diag", "ns_diag"), ("ns_subdomain", "ns_subdomain"),
                         ("ns_batch_config", "ns_batch_config"), ("ns_kernel_time", "ns_kernel_time")):
        cf = cs[cname]
        ff = ft[fname]
        assert [x[0] for x in cf] == [x[0] for x in ff], (cname, cf, ff)
        for (n, ct, ce), (_, fk, fe) in zip(cf, ff):
            assert C2F[ct] == fk, (cname, n, ct, fk)
            assert ce == fe, (cname, n, ce, fe)


def test_c_string_helper_and_module_shape():
    src = open(F90).read()
    assert "module ns_gpu" in src and "end module ns_gpu" in src
    assert "function ns_string(p)" in src
