"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports
every entry point declared in include/*.h; the native host driver builds; the
package has no compute path besides the CUDA library."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(tdvmc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("tdvmc_create", "tdvmc_sample", "tdvmc_eval_local", "tdvmc_eval_local_adjoint", "tdvmc_reduce_stats",
              "tdvmc_tdvp_rhs", "tdvmc_step"):
        assert n in names


def test_library_loads_and_exports_every_declared_symbol():
    from tdvmc_gb300 import _native as N
    lib = N.load()
    for n in declared_functions():
        assert hasattr(lib, n), n
    assert set(N.EXPORTS) <= set(declared_functions()) | set(N.EXPORTS)
    # a compute call without a GPU fails loudly with a CUDA status, never silently
    assert lib.tdvmc_status_string(2).decode() == "CUDA error"


def test_library_is_sm103a():
    from tdvmc_gb300 import build as B
    assert "arch=compute_103a,code=sm_103a" in " ".join(B.ARCH)


def test_host_driver_built():
    from tdvmc_gb300 import build as B
    B.build()
    assert os.path.exists(B.RUNNER) and os.access(B.RUNNER, os.X_OK)


def test_package_does_not_import_the_oracle():
    pkg = os.path.join(ROOT, "tdvmc_gb300")
    for f in glob.glob(os.path.join(pkg, "**", "*.*"), recursive=True):
        if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h", ".inc")):
            text = open(f).read()
            assert "oracle" not in re.sub(r"#.*|//.*", "", text).replace("oracle/", ""), f


def test_no_gpu_create_reports_cuda_error():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except Exception:
        pass
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    with pytest.raises(N.TdvmcError) as e:
        T.BosonsBulk(3, 8, 10, 4.0, 4)
    assert e.value.code == N.ERR_CUDA
