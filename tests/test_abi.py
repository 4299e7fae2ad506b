"""The C-ABI library: every entry point declared in include/b3g.h is exported and bound, and the
library fails loudly (an error code, no CPU fallback) when no GPU is usable."""
import ctypes as C
import os
import re

import pytest
from conftest import ROOT, gpu_available

from bounce_softbody_gb300 import b3g

HEADER = os.path.join(ROOT, "include", "b3g.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"B3G_API\s+[\w\s\*]+?\b(b3g_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(b3g.LIB_PATH)
    names = declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    assert sorted(b3g.SIGNATURES) == declared()


def test_solver_config_defaults_are_the_references():
    c = b3g.SolverConfig()
    b3g.load_library().b3g_solver_config_default(C.byref(c))
    assert c.force_iterations == 1 and c.max_pcg_iterations == 20
    assert abs(c.pcg_tolerance - 1.1920928955078125e-07) < 1e-20
    assert c.refresh_period == 50 and c.precision == 0 and c.preconditioner == 0


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_context_creation_fails_loudly_without_gpu():
    with pytest.raises(b3g.B3gError):
        b3g.Context(0)


def test_null_arguments_are_rejected():
    lib = b3g.load_library()
    assert lib.b3g_body_step(None, C.c_float(0.01), None, None) == 1
    assert lib.b3g_context_create(0, None) == 1
    assert b"null" in lib.b3g_last_error()
