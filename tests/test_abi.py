"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/sdem_gpu.h declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re

from sdem_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "sdem_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(sdem_[a-z_0-9]+)\s*\(", hdr)))


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    assert set(capi.EXPORTED) <= set(syms), set(capi.EXPORTED) - set(syms)


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_cfg_struct_layout_matches_header():
    # sdem_default_cfg is host-only: it fills the struct without touching a GPU
    lib = capi.load(build.build())
    cfg = capi.SdemCfg()
    lib.sdem_default_cfg(ctypes.byref(cfg))
    assert cfg.cntct_list_size == 6 and cfg.base_wall_id == 10000000 and cfg.wall_max_update_iter == 100
    assert cfg.dt == 1.0e-5 and tuple(cfg.gravity) == (0.0, -9.81, 0.0) and cfg.wall_neighbor_ratio == 2.0
    assert cfg.quirk_ab2_rot == 1 and cfg.cs_ratio == 1.0


def test_headers_compile_as_c_and_cxx(tmp_path):
    # a C or C++ host includes the headers as they are (no CUDA headers needed)
    import shutil
    import subprocess
    import pytest
    for cc, lang in (("gcc", "c"), ("g++", "c++")):
        exe = shutil.which(cc)
        if exe is None:
            pytest.skip(f"no {cc}")
        for h in ("sdem_gpu.h", "sdem_surrogate.h"):
            src = tmp_path / f"use_{h}.{'c' if lang == 'c' else 'cpp'}"
            src.write_text(f'#include "{os.path.join(ROOT, "include", h)}"\nint main(void) {{ return 0; }}\n')
            r = subprocess.run([exe, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", lang, str(src)],
                               capture_output=True, text=True)
            assert r.returncode == 0, (cc, h, r.stderr)
