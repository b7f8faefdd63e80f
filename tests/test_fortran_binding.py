"""The Fortran binding (fortran/channel_gpu.f90) against the C header.

No Fortran compiler exists in the build image, so the ISO_C_BINDING module is
checked by reading both files: every function include/channel_gpu.h declares
has exactly one Bind(C) interface of the same name, the same argument count
and order, and argument declarations that pass what the C prototype expects
(scalars by value with the matching kind, arrays and out-arguments by
reference, handles and device pointers as Type(c_ptr) by value), the same
return kind; the Bind(C) cf_params type lists the C struct's fields in order
with matching kinds; and the drop-in module defines the reference's
subroutine names."""
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "channel_gpu.h")
FORTRAN = os.path.join(ROOT, "fortran", "channel_gpu.f90")

HANDLES = {"cf_ctx", "cf_mlp", "cf_ensemble", "void"}


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def c_prototypes():
    """name -> (return kind, [(base, mode)]) from the header, where mode is
    'value', 'ref' (a pointer or array of base) or 'handle' (an opaque handle
    or void pointer passed by value)."""
    text = _strip_c(open(HEADER).read())
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(cf_\w+)\s*\(([^;{}]*?)\)\s*;", text):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef"):
            continue
        params = []
        for a in ([] if args in ("", "void") else args.split(",")):
            a = a.strip()
            arr = re.search(r"\[(\d*)\]\s*$", a)
            a0 = re.sub(r"\[\d*\]\s*$", "", a).strip()
            nm = re.search(r"(\w+)\s*$", a0).group(1)
            ty = a0[: -len(nm)].replace("const", " ").strip()
            stars = ty.count("*") + (1 if arr else 0)
            base = ty.replace("*", " ").split()[-1]
            if base in HANDLES and base != "void":
                mode = "handle" if stars == 1 else "handle_ref"
            elif base == "void":
                mode = "handle"
            elif stars == 0:
                mode = "value"
            else:
                mode = "ref"
            params.append((base, mode, nm))
        r = ret.replace("const", " ").split()
        if r == ["void"]:
            rk = "subroutine"
        elif "*" in ret:
            rk = "ptr"
        else:
            rk = r[-1]
        out[name] = (rk, params)
    return out


F_KIND = {"integer(c_int)": "int", "integer(c_long)": "long", "real(c_double)": "double", "real(c_float)": "float",
          "type(c_ptr)": "ptr", "character(kind=c_char)": "char", "type(cf_params)": "cf_params"}


def fortran_interfaces():
    """name -> (bind name, return kind, [(base, value, is_array)]) of the
    interface blocks of module channel_gpu."""
    text = open(FORTRAN).read()
    text = re.sub(r"!.*", "", text)
    text = re.sub(r"&\s*\n\s*", " ", text)
    mod = text[text.lower().index("module channel_gpu"):text.lower().index("end module channel_gpu")]
    block = mod[mod.lower().index("interface"):mod.lower().index("end interface")]
    out = {}
    hdr = re.compile(r"^\s*(?:(integer\(c_int\)|type\(c_ptr\))\s+)?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*"
                     r"bind\(c,\s*name=\"(\w+)\"\)", re.I | re.M)
    heads = list(hdr.finditer(block))
    for q, m in enumerate(heads):
        body = block[m.end(): heads[q + 1].start() if q + 1 < len(heads) else len(block)]
        body = body[: re.search(r"end\s+(function|subroutine)", body, re.I).start()]
        ret = "subroutine" if m.group(2).lower() == "subroutine" else {"integer(c_int)": "int", "type(c_ptr)": "ptr"}[
            m.group(1).lower()]
        args = [a.strip() for a in m.group(4).split(",") if a.strip()]
        decl = {}
        for line in body.split("\n"):
            line = line.strip()
            if "::" not in line or line.lower().startswith("import"):
                continue
            spec, names = line.split("::", 1)
            parts = [p.strip().lower().replace(" ", "") for p in re.split(r",(?![^()]*\))", spec)]
            kind = F_KIND[parts[0]]
            value = "value" in parts[1:]
            for nm in re.split(r",(?![^()]*\))", names):
                nm = nm.strip()
                a = re.match(r"(\w+)\s*(\(.*\))?$", nm)
                decl[a.group(1).lower()] = (kind, value, a.group(2) is not None)
        params = [decl[a.lower()] for a in args]
        out[m.group(3)] = (m.group(5), ret, params, args)
    return out


def test_every_c_function_has_a_matching_fortran_interface():
    cp = c_prototypes()
    fi = fortran_interfaces()
    assert len(cp) > 60, len(cp)
    assert set(cp) == set(fi), (sorted(set(cp) - set(fi)), sorted(set(fi) - set(cp)))
    for name, (rk, cparams) in cp.items():
        bind, frk, fparams, fargs = fi[name]
        assert bind == name, name
        assert frk == rk if rk in ("subroutine", "ptr") else frk == "int", (name, rk, frk)
        assert len(fparams) == len(cparams), (name, len(cparams), len(fparams))
        for (base, mode, cname), (fk, val, arr), fname in zip(cparams, fparams, fargs):
            where = f"{name}({cname})"
            if mode == "value":
                assert fk == base and val, where
            elif mode == "handle":
                assert fk == "ptr" and val, where
            elif mode == "handle_ref":
                assert fk == "ptr" and not val, where
            elif base == "char":
                assert fk == "char" and not val and arr, where
            elif base == "cf_params":
                assert fk == "cf_params" and not val, where
            else:  # pointer to int/double/float: a Fortran reference, or a device pointer by value
                assert (fk == base and not val) or (fk == "ptr" and val), where


def test_cf_params_layout():
    text = _strip_c(open(HEADER).read())
    body = re.search(r"typedef\s+struct\s*\{(.*?)\}\s*cf_params\s*;", text, re.S).group(1)
    cfields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ty, names = decl.split(None, 1)
        cfields += [(ty, n.strip()) for n in names.split(",")]
    ftext = re.sub(r"!.*", "", open(FORTRAN).read())
    fbody = re.search(r"type,\s*bind\(c\)\s*::\s*cf_params(.*?)end\s+type", ftext, re.S | re.I).group(1)
    ffields = []
    for line in fbody.split("\n"):
        if "::" in line:
            spec, names = line.split("::")
            ffields += [(F_KIND[spec.strip().lower().replace(" ", "")], n.strip()) for n in names.split(",")]
    assert [(t, n.lower()) for t, n in cfields] == [(t, n.lower()) for t, n in ffields]


def test_constants_match():
    text = _strip_c(open(HEADER).read())
    ftext = open(FORTRAN).read()
    for name, val in re.findall(r"\b(CF_[A-Z0-9_]+)\s*=\s*(\d+)", text):
        m = re.search(rf"\b{name}\s*=\s*(\d+)", ftext)
        assert m and m.group(1) == val, name


def test_dropin_module_has_the_reference_subroutines():
    """The subroutines time_integration.f90 calls (and the diagnostics that
    call the path), by the reference's names and dummy-argument counts."""
    text = re.sub(r"!.*", "", open(FORTRAN).read())
    mod = text[text.lower().index("module channel_gpu_dropin"):]
    subs = {}
    for m in re.finditer(r"^\s*subroutine\s+(\w+)\s*(\([^)]*\))?", mod, re.I | re.M):
        args = (m.group(2) or "()")[1:-1]
        subs[m.group(1).lower()] = len([a for a in args.split(",") if a.strip()])
    want = {"compute_time_step_rk3": 0, "compute_dt": 0, "compute_eddy_viscosity": 5, "compute_wall_model": 4,
            "compute_rhs_u": 4, "compute_rhs_v": 4, "compute_rhs_w": 4, "apply_boundary_conditions": 0,
            "compute_projection_step": 0, "compute_dpx_for_constant_mass_flow": 2,
            "compute_dpy_for_constant_mass_flow": 2, "compute_dpx_for_constant_ucenterline": 2,
            "check_divergence": 1, "compute_pressure": 0}
    for k, n in want.items():
        assert subs.get(k) == n, (k, subs.get(k), n)
