"""The C-ABI library: every entry point declared in include/*.h (b3g.h, b3g_sparse.h) is exported
and bound, and the library fails loudly (an error code, no CPU fallback) when no GPU is usable."""
import ctypes as C
import os
import re

import pytest
from conftest import ROOT, gpu_available

from bounce_softbody_gb300 import b3g, b3g_sparse

HEADER = os.path.join(ROOT, "include", "b3g.h")
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared():
    text = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"B3G_API\s+[\w\s\*]+?\b(b3g_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(b3g.LIB_PATH)
    names = declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    assert sorted(set(b3g.SIGNATURES) | set(b3g_sparse.SIGNATURES)) == declared()


def test_solver_config_defaults_are_the_references():
    c = b3g.SolverConfig()
    b3g.load_library().b3g_solver_config_default(C.byref(c))
    assert c.force_iterations == 1 and c.max_pcg_iterations == 20
    assert abs(c.pcg_tolerance - 1.1920928955078125e-07) < 1e-20
    assert c.refresh_period == 50 and c.precision == 0 and c.preconditioner == 0
    assert c.contact_mode == b3g.CONTACT_PENALTY


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_context_creation_fails_loudly_without_gpu():
    with pytest.raises(b3g.B3gError):
        b3g.Context(0)


def test_null_arguments_are_rejected():
    lib = b3g.load_library()
    assert lib.b3g_body_step(None, C.c_float(0.01), None, None) == 1
    assert lib.b3g_context_create(0, None) == 1
    assert b"null" in lib.b3g_last_error()


# ctypes mirror -> C struct of include/b3g.h
MIRRORS = {"WorldShapeC": "b3g_world_shape", "RayHit": "b3g_ray_hit", "BodyDescC": "b3g_body_desc",
           "SolverConfig": "b3g_solver_config", "StepStats": "b3g_step_stats",
           "RequestResult": "b3g_request_result", "ServerStats": "b3g_server_stats",
           "b3g_sparse.SolveCGInput": "b3g_solve_cg_input", "b3g_sparse.SolveCGOutput": "b3g_solve_cg_output",
           "b3g_sparse.ForceSolverData": "b3g_sparse_force_solver_data",
           "b3g_sparse.ForceModelC": "b3g_sparse_force_model", "b3g_sparse.SolveBEInput": "b3g_solve_be_input",
           "b3g_sparse.SolveBEOutput": "b3g_solve_be_output"}


def mirror(name):
    mod, _, cls = name.rpartition(".")
    return getattr(b3g_sparse if mod == "b3g_sparse" else b3g, cls)


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror in b3g.py has the size and field offsets the C compiler gives the
    header's struct (a host binding with a stale layout would pass garbage through the ABI)."""
    import subprocess

    lines = ["#include <cstdio>", "#include <cstddef>", '#include "b3g.h"', '#include "b3g_sparse.h"', "int main() {"]
    for py, c in MIRRORS.items():
        lines.append(f'std::printf("{py} size %zu\\n", sizeof({c}));')
        for f, _ in mirror(py)._fields_:
            lines.append(f'std::printf("{py} {f} %zu\\n", offsetof({c}, {f}));')
    lines += ["return 0; }"]
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for line in filter(None, out):
        py, what, val = line.split()
        cls = mirror(py)
        got = C.sizeof(cls) if what == "size" else getattr(cls, what).offset
        assert got == int(val), (py, what, got, int(val))


def test_enum_values_match_the_header():
    from bounce_softbody_gb300 import meshes

    text = open(HEADER).read()
    enum = {k: int(v) for k, v in re.findall(r"\b(B3G_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    pairs = {"PRECISION_FP32": "B3G_PRECISION_FP32", "PRECISION_FP64": "B3G_PRECISION_FP64",
             "PRECISION_BF16": "B3G_PRECISION_BF16_BLOCKS", "PRECOND_JACOBI": "B3G_PRECOND_JACOBI",
             "PRECOND_BLOCK_JACOBI": "B3G_PRECOND_BLOCK_JACOBI", "CONTACT_PENALTY": "B3G_CONTACT_PENALTY",
             "CONTACT_FILTER": "B3G_CONTACT_FILTER"}
    for py, c in pairs.items():
        assert getattr(b3g, py) == enum[c], py
    shapes = {"SHAPE_SPHERE": "B3G_SHAPE_SPHERE", "SHAPE_CAPSULE": "B3G_SHAPE_CAPSULE", "SHAPE_BOX": "B3G_SHAPE_BOX",
              "SHAPE_TRIANGLE": "B3G_SHAPE_TRIANGLE", "SHAPE_MESH": "B3G_SHAPE_MESH", "SHAPE_SDF": "B3G_SHAPE_SDF"}
    for py, c in shapes.items():
        assert getattr(meshes, py) == enum[c], py
    for code, name in b3g.SOLVE_STATUS.items():
        assert enum["B3G_SOLVE_" + name.upper()] == code, name


def test_integration_c_example_compiles_and_links(tmp_path):
    """The C usage example of the integration guide (tests/integration_example.c) compiles as C
    against include/b3g.h and links against libb3g.so (it is not run: no GPU)."""
    import subprocess

    src = os.path.join(ROOT, "tests", "integration_example.c")
    lib = os.path.dirname(b3g.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-Wno-unused-variable", "-c", "-I",
                        os.path.join(ROOT, "include"), src, "-o", str(tmp_path / "example.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    main = tmp_path / "main.c"
    main.write_text("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", str(tmp_path / "example.o"), str(main), "-L", lib, "-lb3g", "-o", str(tmp_path / "ex")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
