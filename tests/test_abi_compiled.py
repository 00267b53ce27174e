"""include/ktri.h as a C and a C++ compiler see it, and include/katric_shim.hpp (the
drop-in for KaTric's run_shmem / run_local) compiled against a stand-in of KaTric's types.

The ctypes binding (katric_gb300/_native.py) re-declares the ABI structs by hand; the CPU tests
here compile tests/abi/abi_check.c with gcc and tests/abi/shim_check.cpp with g++ against the
header and libktri.so, and check every struct's size and every field's offset against the
ctypes mirror, so a drift in field order or padding fails here.  The GPU tests run the same
programs on the reference's example graphs (binary format, examples/*.first_out / *.head, and
their totals from examples/examples.yaml)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from katric_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ABI = os.path.join(ROOT, "tests", "abi")


@pytest.fixture(scope="module")
def programs(tmp_path_factory):
    if not (shutil.which("gcc") and shutil.which("g++")):
        pytest.skip("gcc/g++ not found")
    lib = build.build()
    libdir = os.path.dirname(lib)
    out = tmp_path_factory.mktemp("abi")
    c_prog, cpp_prog = str(out / "abi_check"), str(out / "shim_check")
    link = [f"-L{libdir}", "-lktri", f"-Wl,-rpath,{libdir}"]
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ABI, "abi_check.c"), "-o", c_prog] + link, check=True)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ABI, "stub"), os.path.join(ABI, "shim_check.cpp"), "-o", cpp_prog] + link,
                   check=True)
    return c_prog, cpp_prog


def _run(args) -> str:
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _layout(text: str) -> dict:
    out = {}
    for line in text.splitlines():
        parts = line.split()
        if len(parts) == 2:
            out[parts[0]] = int(parts[1])
        elif len(parts) == 3:
            out[parts[0]] = (int(parts[1]), int(parts[2]))
    return out


MIRRORS = {"ktri_opts": _native.Opts, "ktri_run_stats": _native.RunStats, "ktri_server_opts": _native.ServerOpts,
           "ktri_server_stats": _native.ServerStats, "ktri_tuning": _native.Tuning}


def test_struct_layouts_match_the_ctypes_mirror(programs):
    c_prog, cpp_prog = programs
    lay = _layout(_run([c_prog, "sizes"]))
    checked = 0
    for key, val in lay.items():
        struct, _, field = key.partition(".")
        mirror = MIRRORS[struct]
        if not field:
            assert ctypes.sizeof(mirror) == val, f"sizeof({struct})"
        else:
            desc = getattr(mirror, field)
            assert (desc.offset, desc.size) == val, f"{struct}.{field}"
        checked += 1
    assert checked > 40
    cpp = _layout(_run([cpp_prog, "sizes"]))
    assert cpp["ktri_opts"] == lay["ktri_opts"] and cpp["ktri_run_stats"] == lay["ktri_run_stats"]


def _write_examples(golden, where) -> dict:
    """The example graphs in the reference's binary format; returns stem -> expected total."""
    ex, _ = golden
    stems = {}
    for g in ex["graphs"]:
        stem = os.path.join(where, g["name"])
        fo = np.array(g.get("binary_first_out", g["first_out"]), dtype="<u8")
        hd = np.array(g.get("binary_head", g["head"]), dtype="<u8")
        fo.tofile(stem + ".first_out")
        hd.tofile(stem + ".head")
        stems[stem] = g["triangles"]
    return stems


@pytest.mark.gpu
def test_c_program_counts_the_examples(programs, golden, tmp_path):
    c_prog, _ = programs
    stems = _write_examples(golden, str(tmp_path))
    out = _run([c_prog, "count"] + list(stems))
    seen = 0
    for line in out.splitlines():
        stem, t1, t2, s = line.split()
        assert int(t1) == int(t2) == stems[stem]
        assert int(s) == 3 * stems[stem]
        seen += 1
    assert seen == len(stems) == 3


@pytest.mark.gpu
def test_shim_counts_like_run_shmem_and_run_local(programs, golden, tmp_path):
    _, cpp_prog = programs
    stems = _write_examples(golden, str(tmp_path))
    for stem, expect in stems.items():
        t_auto, t_merge, s, t_local = (int(x) for x in _run([cpp_prog, "count", stem]).split())
        assert t_auto == t_merge == t_local == expect, stem
        assert s == 3 * expect
