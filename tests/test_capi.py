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


def test_mirrored_system_descriptor_checks():
    """NUBosonsBulkPB descriptors that the reference could not run are refused
    before any device call: no knots (it reads r_max from them), a potential other
    than its square well, knots so short that a mirrored distance 2 r_max - r
    could turn negative, and an unknown system type."""
    import ctypes as C
    import numpy as np
    from tdvmc_gb300 import _native as N
    lib = N.load()

    def create(system_type=N.SYS_NU_BOSONS_BULK_PB, knots=(0.0, 0.5, 1.0, 1.5, 2.0), pot=N.POT_SQUARE, L=4.0,
               dim=3):
        d = N.SystemDesc()
        d.dim, d.n, d.p = dim, 8, 5
        kn = None if knots is None else np.ascontiguousarray(knots, dtype=np.float64)
        d.n_user_knots = 0 if kn is None else kn.size
        d.user_knots = C.POINTER(C.c_double)() if kn is None else kn.ctypes.data_as(C.POINTER(C.c_double))
        d.box_length, d.pot_kind, d.n_pot = L, pot, 2
        d.pot[0], d.pot[1] = 0.5, 1.0
        d.hbar2_2m, d.precision, d.system_type, d.n_walkers = 1.0, N.PREC_FP64, system_type, 4
        h = C.c_void_p()
        rc = lib.tdvmc_create(C.byref(d), C.byref(h))
        if rc == 0:
            lib.tdvmc_destroy(h)
        return rc

    assert create(knots=None) == N.ERR_ARG
    assert create(pot=N.POT_LJ) == N.ERR_ARG
    # 3D, L = 4: the largest minimum-image distance is 2 sqrt(3) = 3.46, so r_max must reach 1.73
    assert create(knots=(0.0, 0.4, 0.8, 1.2, 1.6)) == N.ERR_ARG
    assert create(system_type=7) == N.ERR_ARG
    # 1D: r_max = L / 4 + 0.4 is enough
    assert create(knots=(0.0, 0.35, 0.7, 1.05, 1.4), dim=1) != N.ERR_ARG
    assert create(knots=(0.0, 0.35, 0.7, 1.05, 1.4), dim=1, system_type=N.SYS_NU_BOSONS_BULK_PB_EXACT) != N.ERR_ARG


def test_header_compiles_as_c_and_matches_the_ctypes_layout(tmp_path):
    """The header is plain C99 (no C++ types cross the boundary), and the struct
    layouts the Python binding declares match the compiler's: size and the offset
    of every field of tdvmc_system_desc, tdvmc_stats, tdvmc_step_opts and
    tdvmc_drops_desc."""
    import ctypes as C
    import shutil
    import subprocess
    from tdvmc_gb300 import _native as N
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"tdvmc_system_desc": N.SystemDesc, "tdvmc_stats": N.Stats, "tdvmc_step_opts": N.StepOpts,
               "tdvmc_drops_desc": N.DropsDesc}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "tdvmc_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%%s size %%zu\\n", "%s", sizeof(%s));' % (cname, cname))
        for f in py._fields_:
            lines.append('printf("%%s %%s %%zu\\n", "%s", "%s", offsetof(%s, %s));' % (cname, f[0], cname, f[0]))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I" + os.path.join(ROOT, "include"),
                           str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])
