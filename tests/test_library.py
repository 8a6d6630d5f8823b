"""CPU tests of the C-ABI library: it loads, exports every function that
include/nl2d_gpu.h declares, and reports errors instead of crashing when no
GPU is usable.  No compute call runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

import nl2d_testlib as T

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "nl2d_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", src)) -
                  {"defined", "if"})


@pytest.fixture(scope="module")
def lib():
    import psyclonebench_gb300 as P
    from psyclonebench_gb300 import build
    if not os.path.exists(P.LIB_PATH):
        build.build()
    return P.load_library()


def test_header_lists_expected_entry_points():
    names = declared_functions()
    for must in ("c_invoke_time_step", "c_read_from_device", "c_write_to_device"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    import psyclonebench_gb300 as P
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in P.EXPORTS, "binding missing for %s" % name


def test_no_gpu_is_an_error_not_a_crash(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import psyclonebench_gb300 as P
    m = T.make_model(12, 12, 1)
    args = m.step_args(0)
    del args[25]
    rc = lib.nl2d_register(*args)
    assert rc == P.NL2D_ERR_CUDA
    buf = ctypes.create_string_buffer(256)
    assert lib.nl2d_last_error(buf, 256) in (P.NL2D_OK, P.NL2D_ERR_CUDA)
    out = np.zeros(3)
    assert lib.nl2d_checksums(T.dptr(out)) == P.NL2D_ERR_STATE
    assert lib.nl2d_last_error(buf, 256) == P.NL2D_ERR_STATE  # message kept until read
    assert lib.nl2d_set_mode(7) == 0  # unknown mode: kept, error recorded
    assert lib.nl2d_last_error(buf, 256) == P.NL2D_ERR_ARGS


def test_missing_library_fails_loudly(tmp_path):
    import psyclonebench_gb300 as P
    saved = P._lib
    P._lib = None
    try:
        with pytest.raises(P.Nl2dError):
            P.load_library(str(tmp_path / "nope.so"))
    finally:
        P._lib = saved


def test_checkpoint_needs_a_problem(lib, tmp_path):
    """Without a registered problem both checkpoint calls report
    NL2D_ERR_STATE and touch no GPU."""
    import psyclonebench_gb300 as P
    path = str(tmp_path / "ck.bin").encode()
    ist = ctypes.c_int(0)
    assert lib.nl2d_checkpoint_write(path, 1) == P.NL2D_ERR_STATE
    assert lib.nl2d_checkpoint_read(path, ctypes.byref(ist)) == P.NL2D_ERR_STATE
    buf = ctypes.create_string_buffer(256)
    lib.nl2d_last_error(buf, 256)


def test_exact_helpers_keep_bit_work_off_the_fp64_pipe():
    """The exact FP64 helpers move a double's bit pattern through inline
    PTX, not a bitcast: through a bitcast the compiler rewrote their integer
    tests as FP64 abs / compare / copysign instructions (on GB300's narrow
    FP64 pipe: 21-27 % of the FP64 step's and the tracer's time).  A source
    check, since the bits are identical either way and only the instruction
    count shows the difference."""
    csrc = os.path.join(REPO, "psyclonebench_gb300", "csrc")
    src = open(os.path.join(csrc, "nl2d_exact.cuh")).read()
    body = lambda name: re.search(r"\b%s\([^)]*\)\s*\{(.*?)\n\}" % name, src, re.S).group(1)
    for name in ("bits", "from_bits"):
        b = body(name)
        assert "mov.b64" in b and "asm(" in b, name
        assert "__double_as_longlong" not in b and "__longlong_as_double" not in b, name
    for f in ("nl2d_fused_tile.cuh", "tra_adv.cu", "nl2d_intfp.cuh"):
        text = open(os.path.join(csrc, f)).read()
        assert "__double_as_longlong" not in text and "__longlong_as_double" not in text, f
