"""The C ABI library loads without a GPU and exports every function that
include/rsg.h declares; the Python binding declares exactly those."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rsg.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:rsg_status|int32_t|int64_t|const char\*)\s+(rsg_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from ressim_gb300 import build

    if not os.path.exists(build.LIB):
        try:
            build.build()
        except FileNotFoundError:
            pytest.skip("nvcc not available to build libresgpu.so")
    return C.CDLL(build.LIB)


def test_header_declares_the_api():
    names = declared()
    for must in ("rsg_context_create", "rsg_csr_create", "rsg_solver_solve", "rsg_mesh_compute_mpfa", "rsg_sim_step",
                 "rsg_cg_diagonal_noalloc"):
        assert must in names
    assert len(names) >= 50


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_matches_header(lib):
    from ressim_gb300 import api

    src = open(api.__file__).read()
    bound = set(re.findall(r'"(rsg_\w+)":', src))
    assert bound == set(declared())


def test_abi_version_and_status_strings(lib):
    lib.rsg_abi_version.restype = C.c_int32
    assert lib.rsg_abi_version() == 1
    lib.rsg_status_string.restype = C.c_char_p
    assert lib.rsg_status_string(3) == b"NOT_CONVERGED_BREAKDOWN"


def test_context_fails_loudly_without_gpu(lib):
    # no CPU fallback: without a usable GPU the context cannot be created
    import ctypes

    h = ctypes.c_void_p()
    lib.rsg_context_create.restype = C.c_int32
    st = lib.rsg_context_create(0, ctypes.byref(h))
    if st == 0:
        lib.rsg_context_destroy(h)
        pytest.skip("a GPU is present")
    assert st == 10  # RSG_CUDA_ERROR


def test_status_codes_match_the_header(lib):
    from ressim_gb300 import abi

    text = open(HEADER).read()
    start = text.index("RSG_OK = 0")
    block = text[start:text.index("};", start)]  # the status enum
    codes = {int(v): k for k, v in re.findall(r"\bRSG_(\w+)\s*=\s*(\d+)", block)}
    assert codes == abi.STATUS
    lib.rsg_status_string.restype = C.c_char_p
    for code, name in abi.STATUS.items():
        assert getattr(abi, name) == code
        assert lib.rsg_status_string(code).decode() == name


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes structure in ressim_gb300.abi has the size and field
    offsets of the C struct of the same name (compiled against rsg.h)."""
    from ressim_gb300 import abi

    structs = {n: t for n, t in vars(abi).items()
               if n.startswith("rsg_") and isinstance(t, type) and issubclass(t, C.Structure)}
    assert "rsg_adjoint_info" in structs and "rsg_runspec" in structs
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rsg.h"', "int main(void) {"]
    for name, t in sorted(structs.items()):
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for f in t._fields_:  # a trailing "_" avoids a Python keyword (lambda_)
            lines.append(f'  printf("{name} {f[0]} %zu\\n", offsetof({name}, {f[0].rstrip("_")}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            name, field, value = line.split()
            got[(name, field)] = int(value)
    for name, t in structs.items():
        assert got[(name, "size")] == C.sizeof(t), name
        for f in t._fields_:
            assert got[(name, f[0])] == getattr(t, f[0]).offset, (name, f[0])


# entry points that take no handle, or whose null-argument behaviour is not
# RSG_BAD_ARG (checked separately below)
_NO_HANDLE = {"rsg_abi_version", "rsg_sweep_mode", "rsg_status_string", "rsg_context_create", "rsg_host_free",
              "rsg_context_last_error", "rsg_context_kernel_launches"}


def test_null_arguments_are_rejected(lib):
    """Every entry point that takes a handle or output pointer returns
    RSG_BAD_ARG for null arguments (zero counts, zero tolerances) before it
    touches the GPU, so a binding's mistakes surface as statuses, never as
    crashes."""
    from ressim_gb300 import abi, api

    L = api.lib()
    checked = []
    for name in declared():
        if name in _NO_HANDLE:
            continue
        f = getattr(L, name)
        args = []
        for t in f.argtypes:
            if t in (C.c_int32, C.c_int64, C.c_size_t):
                args.append(0)
            elif t is C.c_double:
                args.append(0.0)
            else:
                args.append(None)
        if name in ("rsg_ensemble_step", "rsg_ensemble_step_batched", "rsg_solver_solve_batched"):
            args[0] = 1  # one member, given as a null array
        assert f(*args) == abi.BAD_ARG, name
        checked.append(name)
    assert len(checked) >= 55
    assert L.rsg_context_last_error(None) == b""
    assert L.rsg_context_kernel_launches(None) == 0
    assert L.rsg_host_free(None) == abi.OK


def test_pointer_helpers_reject_wrong_arrays():
    """Arrays handed to the C ABI are checked for type and layout even under
    python -O."""
    import numpy as np

    from ressim_gb300 import abi

    with pytest.raises(TypeError):
        abi.dptr(np.zeros(3, np.float32))
    with pytest.raises(TypeError):
        abi.iptr(np.zeros(3, np.int64))
    with pytest.raises(TypeError):
        abi.dptr(np.zeros((4, 4))[:, 0])
    keep = abi.Keep()
    with pytest.raises(ValueError):
        abi.table(keep, [np.arange(3.0)], np.zeros(4))
    with pytest.raises(ValueError):
        abi.even_table(keep, [(0.0, 1.0), (0.0, 1.0)], np.zeros(4))
