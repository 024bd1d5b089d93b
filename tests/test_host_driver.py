"""CPU tests of the native host driver's control logic (tdvmc_run), linked
against a CPU stand-in of the C ABI (tests/host/fake_capi.cpp): the
CONFIG_VERSION check (TDVMC.cpp:3039-3043), the coordinate files read at the
start and written at the end (TDVMC.cpp:640-670, 4010-4018), the final config
(TDVMC.cpp:4027-4034), and the parameter-acceptance trials with the 5-step
set-back (TDVMC.cpp:2585-2630, 2746-2784, 3648-3916)."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("fakebuild")
    exe = str(d / "tdvmc_run_fake")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tdvmc_gb300", "csrc", "host", "tdvmc_run.cpp"),
                           os.path.join(ROOT, "tests", "host", "fake_capi.cpp"), "-o", exe])
    return exe


def base_cfg(**kw):
    c = {"CONFIG_VERSION": "0.24", "SYSTEM_TYPE": "BosonsBulk", "N": 8, "LBOX": 2.0, "DIM": 3, "N_PARAM": 4,
         "MC_STEP": 0.3, "MC_NSTEPS": 4, "MC_NTHERMSTEPS": 16, "MC_VERY_FIRST_NINITIALIZATIONSTEPS": 5,
         "TIMESTEP": 0.01, "TOTALTIME": 0.095, "IMAGINARY_TIME": 0, "ODE_SOLVER_TYPE": 2,
         "WRITE_EVERY_NTH_STEP_TO_FILE": 1, "SYSTEM_PARAMS": [0.5, 1.0], "PARAMS_REAL": [1.0, 1.0, 1.0, 1.0],
         "PARAMS_IMAGINARY": [0.0], "PARAM_PHIR": 0.0, "PARAM_PHII": 0.0}
    c.update(kw)
    return c


def run(driver, tmp_path, cfg, env=None, coords=None):
    cdir = tmp_path / "cfg"
    cdir.mkdir(exist_ok=True)
    if coords is not None:
        (cdir / "coords").mkdir(exist_ok=True)
        for k, line in enumerate(coords):
            (cdir / "coords" / ("particleconfiguration_8_3D_%d.csv" % k)).write_text("junk\n" + line + "\n")
    path = cdir / "run.config"
    path.write_text(json.dumps(cfg))
    out = tmp_path / "out"
    log = tmp_path / "fake.log"
    e = dict(os.environ, FAKE_LOG=str(log), **(env or {}))
    r = subprocess.run([driver, str(path), str(out)], capture_output=True, text=True, env=e)
    return r, out, (log.read_text().splitlines() if log.exists() else [])


def table(path):
    return np.loadtxt(path, skiprows=1, ndmin=2)


def test_config_version_is_checked(driver, tmp_path):
    r, _, _ = run(driver, tmp_path, base_cfg(CONFIG_VERSION="0.23"))
    assert r.returncode == 1 and "out of date" in r.stderr


def test_plain_run_and_end_files(driver, tmp_path):
    r, out, log = run(driver, tmp_path, base_cfg())
    assert r.returncode == 0, r.stderr
    E = table(out / "AllLocalEnergyR.dat")[:, 0]
    assert list(E) == list(range(1, 11))  # 10 steps, one trial each
    assert sum(1 for l in log if l.startswith("step")) == 10
    fin = json.loads((out / "AAFinish_tVMC.config").read_text())
    uR = np.asarray(fin["PARAMS_REAL"])
    assert np.allclose(uR, 1.0 + 0.01 * sum(range(1, 11)))
    assert fin["CONFIG_VERSION"] == "0.24" and fin["N"] == 8
    pos = np.loadtxt(out / "AAFinish_particleconfiguration_8_3D.dat")
    assert pos.size == 24
    assert (out / "coords" / "particleconfiguration_8_3D_0.dat").exists()


def test_walkers_start_from_coordinate_files(driver, tmp_path):
    lines = [",".join("%.17g" % (0.01 * (k + 1) * i) for i in range(24)) for k in range(2)]
    r, out, log = run(driver, tmp_path, base_cfg(TOTALTIME=0.0), coords=lines)
    assert r.returncode == 0, r.stderr
    assert "from 2 file(s)" in r.stdout
    # walker 0 takes file 0: its first coordinate (particle 0, x) is 0.0; the data
    # written at the end is the walkers the (fake) library holds
    pos = np.loadtxt(out / "AAFinish_particleconfiguration_8_3D.dat")
    expect = np.array([0.01 * i for i in range(24)])
    assert np.allclose(pos, expect)


def test_rejected_step_retries_then_sets_back_five_steps(driver, tmp_path):
    # call 7 (step 7) is not positive definite; its second trial (call 8) passes, and
    # the reference then sets the run back 5 steps
    cfg = base_cfg(USE_PARAMETER_ACCEPTANCE_CHECK=1, PARAMETER_ACCEPTANCE_CHECK_TYPE=0, TOTALTIME=0.095)
    r, out, log = run(driver, tmp_path, cfg, env={"FAKE_NOT_PD": "7"})
    assert r.returncode == 0, r.stderr
    assert "SetBackNSteps(5)" in r.stderr
    steps = [l for l in log if l.startswith("step")]
    # the retried call used twice the moves
    assert steps[6].endswith("moves 16") and steps[7].endswith("moves 32")
    E = table(out / "AllLocalEnergyR.dat")[:, 0]
    # steps 1-6 recorded, step 7 (trial 2, energy 8) recorded then 5 records dropped:
    # 1, 2 remain, then the run continues from step 3 with calls 9, 10, ...
    assert list(E[:3]) == [1, 2, 9]
    assert len(E) == 10
    # the walkers restarted from their initial configuration with the thermalisation moves
    assert sum(1 for l in log if l.startswith("set_walkers")) == 2
    assert sum(1 for l in log if l.startswith("sample 5 ")) == 2
    # parameters restored to the start of the third step: 1 + 0.01 * (1 + 2)
    sets = [float(l.split()[1]) for l in log if l.startswith("set_params")]
    assert any(abs(v - (1.0 + 0.01 * 3)) < 1e-12 for v in sets)


def test_check_type_2_rejects_large_changes(driver, tmp_path):
    cfg = base_cfg(USE_PARAMETER_ACCEPTANCE_CHECK=1, PARAMETER_ACCEPTANCE_CHECK_TYPE=2, TOTALTIME=0.025)
    r, out, log = run(driver, tmp_path, cfg, env={"FAKE_BIG": "2"})
    assert r.returncode == 0, r.stderr
    assert "PARAMETERS NOT ACCEPTED" in r.stderr
    # type 0 accepts the same change
    r0, _, _ = run(driver, tmp_path, dict(cfg, PARAMETER_ACCEPTANCE_CHECK_TYPE=0), env={"FAKE_BIG": "2"})
    assert "PARAMETERS NOT ACCEPTED" not in r0.stderr


def test_unimplemented_check_type_is_refused(driver, tmp_path):
    r, _, _ = run(driver, tmp_path, base_cfg(USE_PARAMETER_ACCEPTANCE_CHECK=1, PARAMETER_ACCEPTANCE_CHECK_TYPE=3))
    assert r.returncode == 2 and "PARAMETER_ACCEPTANCE_CHECK_TYPE 3" in r.stderr


@pytest.mark.parametrize("fixture", ["driver_d3_n27", "driver_pb_d3_n27"])
def test_output_files_have_the_reference_layout(driver, tmp_path, fixture):
    """The driver on the configs of tests/golden/driver_d3_n27 (BosonsBulk) and
    driver_pb_d3_n27 (NUBosonsBulkPB), the reference's own program run on them
    (tests/golden/make_golden.py): every file the fixture holds comes out with
    the same header line, the same number of rows and columns, and every number
    in the reference's 24-wide %.15e layout (Utils.cpp:809-858); the
    start-parameter files equal the reference's."""
    import re
    gold = os.path.join(ROOT, "tests", "golden", fixture)
    cfg = json.load(open(os.path.join(gold, "run.config")))
    r, out, _ = run(driver, tmp_path, cfg)
    assert r.returncode == 0, r.stderr
    num = re.compile(r"^( {2,3}-?\d\.\d{15}e[+-]\d{2})+$")
    for name in sorted(os.listdir(gold)):
        if not name.endswith(".dat"):
            continue
        ref = open(os.path.join(gold, name)).read().splitlines()
        got = open(out / name).read().splitlines()
        assert len(got) == len(ref), name
        has_header = name != "timesSystem.dat"
        if has_header:
            assert got[0] == ref[0], (name, got[0], ref[0])
        for a, b in zip(got[int(has_header):], ref[int(has_header):]):
            assert num.match(a) and len(a) == len(b), (name, a, b)
    for name in ("ParametersR0.dat", "ParametersI0.dat", "times.dat"):
        assert (out / name).exists(), name
    assert open(out / "ParametersR0.dat").read().splitlines()[0] == "uR_k..."
    p0 = np.loadtxt(out / "ParametersR0.dat", skiprows=1)
    assert np.array_equal(p0, np.asarray(cfg["PARAMS_REAL"]))
    assert open(out / "AllParametersR.dat").read().splitlines()[0] == "%24s%24s" % ("uR_k", "...")
    assert open(out / "AllLocalEnergyR.dat").read().splitlines()[0] == "ER"


def test_mirrored_distance_system(driver, tmp_path):
    """SYSTEM_TYPE NUBosonsBulkPB (TDVMC.cpp:2953-2960): the descriptor carries the
    system type and its square well whatever POTENTIAL says; GPU_PB_EXACT_DERIVATIVES
    switches to the exact form; OtherExpectationValues rows carry 9 + GR_BIN_COUNT
    values, the g(r) entries zero as the reference leaves them."""
    cfg = base_cfg(SYSTEM_TYPE="NUBosonsBulkPB", USE_NURBS=1, NURBS_GRID=[0.0, 0.4, 0.7, 1.0],
                   POTENTIAL="lj", GR_BIN_COUNT=12)
    r, out, log = run(driver, tmp_path, cfg)
    assert r.returncode == 0, r.stderr
    assert "create system 1 pot 1" in log
    other = table(out / "OtherExpectationValues.dat")
    assert other.shape == (10, 9 + 12)
    assert np.all(other[:, 9:] == 0.0)
    r, out, log = run(driver, tmp_path, dict(cfg, GPU_PB_EXACT_DERIVATIVES=1, GR_BIN_COUNT=0))
    assert r.returncode == 0, r.stderr
    assert "create system 2 pot 1" in log
    assert table(out / "OtherExpectationValues.dat").shape[1] == 9 + 400
    r, _, _ = run(driver, tmp_path, base_cfg(SYSTEM_TYPE="NUBosonsBulkPBBox"))
    assert r.returncode == 2
    r, _, _ = run(driver, tmp_path, base_cfg(SYSTEM_TYPE="NUBosonsBulkPB"))  # no knots
    assert r.returncode == 2 and "USE_NURBS" in r.stderr


def test_random_state_for_a_successive_run(driver, tmp_path):
    """random/state_philox.dat (the counterpart of the reference's random/state_*
    files, Utils.cpp:48-78, TDVMC.cpp:515-525, 3958-3964): a run writes its seed
    and epoch; a run that finds the file in its config directory keeps the seed
    and takes the next epoch, so its Philox streams (key = epoch << 32 | seed)
    are new ones."""
    import shutil
    cfg = base_cfg(GPU_SEED=7)
    r, out, log = run(driver, tmp_path, cfg)
    assert r.returncode == 0, r.stderr
    assert (out / "random" / "state_philox.dat").read_text().split() == ["7", "0"]
    assert any(l.startswith("sample 5 seed 7") for l in log)
    (tmp_path / "cfg" / "random").mkdir()
    shutil.copy(out / "random" / "state_philox.dat", tmp_path / "cfg" / "random" / "state_philox.dat")
    (tmp_path / "fake.log").unlink()
    r, out, log = run(driver, tmp_path, cfg)
    assert r.returncode == 0, r.stderr
    assert any(l.startswith("sample 5 seed %d" % ((1 << 32) | 7)) for l in log), log[:5]
    assert (out / "random" / "state_philox.dat").read_text().split() == ["7", "1"]
