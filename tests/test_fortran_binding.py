"""The Fortran side of the drop-in, checked without a Fortran compiler.

- sdem_gb300/fortran/Prtcl_GPU.f90 binds every entry point of
  include/sdem_gpu.h: the same names, the same argument counts, and
  argument passing that matches the C types (a C scalar is passed by value;
  a handle or device/stream address is type(c_ptr) by value; every other C
  pointer is passed by reference).  Its bind(C) struct has the fields of
  struct sdem_cfg in order with matching kinds.
- sdem_gb300/fortran/Prtcl_DEMSystem_gpu.patch is an insertion-only unified
  diff: every hunk adds lines and removes none, each #ifdef SDEM_GPU is
  closed, and it calls only procedures the driver module makes public.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FDIR = os.path.join(ROOT, "sdem_gb300", "fortran")


def c_declarations():
    hdr = open(os.path.join(ROOT, "include", "sdem_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    out = {}
    for m in re.finditer(r"(?:^|\n)\s*(?:int|void|const char\*)\s+(sdem_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", hdr):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = params
    return out


def f_interfaces():
    src = open(os.path.join(FDIR, "Prtcl_GPU.f90")).read()
    src = re.sub(r"!.*", "", src)
    src = re.sub(r"&\s*\n\s*", " ", src)
    out = {}
    for m in re.finditer(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end\s+(?:function|subroutine)",
                         src, flags=re.S | re.I):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        decls = {}
        for line in m.group(4).splitlines():
            if "::" not in line:
                continue
            spec, names = line.split("::", 1)
            for nm in re.findall(r"(\w+)\s*(?:\([^)]*\))?", names):
                decls[nm] = spec.lower()
        out[m.group(3)] = (m.group(1), args, decls)
    return out


def test_every_entry_point_is_bound_with_matching_arguments():
    cdecl = c_declarations()
    fint = f_interfaces()
    assert set(cdecl) == set(fint), (set(cdecl) ^ set(fint))
    for name, params in cdecl.items():
        fname, args, decls = fint[name]
        assert fname == name, name
        assert len(args) == len(params), (name, args, params)
        for a, p in zip(args, params):
            spec = decls[a]
            by_value = "value" in spec
            is_ptr = "*" in p
            if not is_ptr:
                assert by_value, f"{name}: {a} ({p}) must be passed by value"
            elif by_value:
                assert "c_ptr" in spec and p.count("*") == 1, f"{name}: {a} ({p}) by value must be a c_ptr"
            ctype = p.replace("const", "").split()[0]
            if not is_ptr:
                want = {"int": "c_int", "double": "c_double", "long": "c_long_long", "unsigned": "c_long_long"}[ctype]
                assert want in spec, (name, a, p, spec)


def test_cfg_struct_fields_in_order():
    hdr = open(os.path.join(ROOT, "include", "sdem_gpu.h")).read()
    body = re.search(r"typedef struct sdem_cfg \{(.*?)\} sdem_cfg;", hdr, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    cfields = []
    for line in body.split(";"):
        line = line.strip()
        if not line:
            continue
        ty, names = line.split(None, 1)
        for nm in names.split(","):
            nm = nm.strip()
            mm = re.match(r"(\w+)(\[(\d+)\])?", nm)
            cfields.append((mm.group(1), "c_int" if ty == "int" else "c_double", int(mm.group(3) or 1)))
    src = open(os.path.join(FDIR, "Prtcl_GPU.f90")).read()
    tbody = re.search(r"type, bind\(C\) :: sdem_cfg(.*?)end type sdem_cfg", src, flags=re.S).group(1)
    ffields = []
    for line in tbody.strip().splitlines():
        spec, names = line.split("::")
        kind = "c_int" if "c_int" in spec else "c_double"
        for nm in names.split(","):
            mm = re.match(r"\s*(\w+)(\((\d+)\))?", nm)
            ffields.append((mm.group(1), kind, int(mm.group(3) or 1)))
    assert cfields == ffields


def test_patch_inserts_only_and_calls_the_driver():
    text = open(os.path.join(FDIR, "Prtcl_DEMSystem_gpu.patch")).read()
    diff = text[text.index("--- "):]
    hunks = re.findall(r"@@ -(\d+),0 \+(\d+)(?:,(\d+))? @@\n((?:\+.*\n?)*)", diff)
    assert len(hunks) == 6
    added = 0
    for old, new, cnt, body in hunks:
        lines = [ln for ln in body.splitlines() if ln]
        assert all(ln.startswith("+") for ln in lines)
        assert len(lines) == int(cnt or 1)
        assert int(new) == int(old) + 1 + added   # insertion points shift by the lines added before
        added += len(lines)
    assert not re.search(r"^-(?!--)", diff, flags=re.M), "the patch removes a line"
    body = "\n".join(h[3] for h in hunks)
    assert body.count("#ifdef SDEM_GPU") == 5 and body.count("#endif") == 5 and body.count("#else") == 1
    drv = open(os.path.join(FDIR, "Prtcl_GPU_Driver.f90")).read()
    public = set(re.findall(r"\b(gpu_\w+)", re.search(r"public ::(.*?)\n\s*\n", drv, flags=re.S).group(1)))
    called = set(re.findall(r"call (gpu_\w+)", body))
    assert called and called <= public, called - public


def test_patch_applies_to_the_published_file(tmp_path):
    # the insertion points exist as the patch expects them in the
    # reference's Prtcl_DEMSystem.f90 (a dry run of patch on a copy; skipped
    # where the reference's sources or the patch tool are absent)
    import shutil
    import subprocess
    import pytest
    src = os.environ.get("SDEM_REFERENCE_SRC", "/root/reference/src/DEM")
    target = os.path.join(src, "Prtcl_DEMSystem.f90")
    if not os.path.exists(target) or shutil.which("patch") is None:
        pytest.skip("no reference source or no patch tool here")
    shutil.copy(target, tmp_path / "Prtcl_DEMSystem.f90")
    with open(os.path.join(FDIR, "Prtcl_DEMSystem_gpu.patch")) as f:
        r = subprocess.run(["patch", "-p0", "--dry-run"], stdin=f, cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout.lower()
    assert "failed" not in out and "fuzz" not in out and "offset" not in out, r.stdout
