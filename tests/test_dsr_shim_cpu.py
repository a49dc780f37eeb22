"""The boundary as compiled code: a C99 program against include/dsrg.h linked with libdsrg.so, and
the C++ dsr::gpu shim (dfpsr_gb300/dsr) compiled against the reference's own headers.

The shim test builds the reference's models, textures, images and cameras with the reference's API
and draws each case twice, with the reference's renderer and through dsr::gpu, comparing the
images byte for byte: model_render at 800x600 with 20,000 triangles, BGRA/ARGB targets of odd size,
prefilled, colour-only and depth-only targets, a two-part model with diffuse and light maps, an
alpha-filtered model, an orthogonal camera, model_renderDepth, and a renderer frame with a box
occluder, tasks, single triangles, occluders from the triangles given so far, a box test, an
alpha-filtered task and the debug wireframe, plus the reference's call-order error.  Here dsr::gpu
calls an oracle-backed test double of the C ABI (tests/shim/oracle_dsrg.cpp), so the comparison
shows that the shim hands the ABI what the reference holds; the GPU behind the same ABI is held to
the oracle by the GPU tests.  The shim linked with the real libdsrg.so is run too: on a machine
without a GPU its first call must raise the reference's exception type with the library's message.
The reference's sources are needed and exist only where the reference was checked out.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "shim")


def _header_entry_points():
    text = open(os.path.join(ROOT, "include", "dsrg.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*|void \*)\s*(dsrg_\w+)\(", text, re.M)))


def test_c_program_compiles_and_links_against_the_header_and_library(built, tmp_path):
    src = os.path.join(SHIM, "abi_check.c")
    named = set(re.findall(r"\(any_function\)(dsrg_\w+)", open(src).read()))
    assert set(_header_entry_points()) == named  # the program takes every declared entry point by address
    exe = str(tmp_path / "abi_check")
    lib_dir = os.path.join(ROOT, "dfpsr_gb300")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), src,
                           os.path.join(lib_dir, "libdsrg.so"), f"-Wl,-rpath,{lib_dir}", "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert re.match(r"entries \d+ missing 0 context_create (0|2)", out.stdout), out.stdout


@pytest.fixture(scope="module")
def shim_build(built, tmp_path_factory):
    from dfpsr_gb300 import build as b
    from oracle import ref
    source = os.path.join(ref.REFERENCE_ROOT, "Source")
    if not (os.path.isdir(os.path.join(source, "DFPSR")) and ref.available("exact")):
        pytest.skip("the reference's sources are not on this machine")
    out = tmp_path_factory.mktemp("shim")
    shim = b.build_shim(source, str(out))
    flags = ["-std=c++14", "-O2", "-DNDEBUG", "-ffp-contract=off", "-fPIC", "-I", source, "-I", os.path.join(ROOT, "include"),
             "-I", os.path.join(ROOT, "dfpsr_gb300", "dsr"), "-I", os.path.join(ROOT, "oracle")]
    check = str(out / "shim_check.o")
    double = str(out / "oracle_dsrg.o")
    subprocess.check_call(["g++", *flags, "-c", os.path.join(SHIM, "shim_check.cpp"), "-o", check])
    subprocess.check_call(["g++", *flags, "-c", os.path.join(SHIM, "oracle_dsrg.cpp"), "-o", double])
    ref_lib = ref.lib_path("exact")
    oracle_dir = os.path.join(ROOT, "oracle")
    with_double = str(out / "shim_with_oracle")
    subprocess.check_call(["g++", "-o", with_double, check, shim, double, os.path.join(oracle_dir, "liboracle.so"), ref_lib,
                           f"-Wl,-rpath,{oracle_dir}:{os.path.dirname(ref_lib)}", "-lpthread"])
    lib_dir = os.path.join(ROOT, "dfpsr_gb300")
    with_library = str(out / "shim_with_libdsrg")
    subprocess.check_call(["g++", "-o", with_library, check, shim, os.path.join(lib_dir, "libdsrg.so"), ref_lib,
                           f"-Wl,-rpath,{lib_dir}:{os.path.dirname(ref_lib)}", "-lpthread"])
    return with_double, with_library


def test_shim_draws_what_the_reference_draws(shim_build):
    out = subprocess.run([shim_build[0], "compare"], capture_output=True, text=True, timeout=600)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "all equal" in out.stdout
    assert out.stdout.count(": colour equal, depth equal") == 9


def test_shim_linked_with_the_library_reports_through_throw_error(shim_build):
    out = subprocess.run([shim_build[1], "context"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    import torch
    if torch.cuda.is_available():
        assert "created" in out.stdout
    else:
        assert "threw: dsr::gpu: no GPU context on device 0" in out.stdout
