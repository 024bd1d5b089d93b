"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the harness built by ``oracle/ref/build_ref.sh`` (the unmodified
reference C++ sources of mathiasgartner/TDVMC linked with
``oracle/ref/harness.cpp``) on seeded inputs and stores inputs and reference
outputs as ``.npz`` files.  Needs the reference checkout (default
``/root/reference``); the fixtures are committed so the tests never need it.

    python tests/golden/make_golden.py [/path/to/reference] [obs | driver | pb]

The driver fixture (``driver_d3_n27/``) holds the output files of the
reference's full program on a small config, for the host driver's file
format and values.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def fmt(a):
    return " ".join("%.17g" % v for v in np.asarray(a, dtype=np.float64).reshape(-1))


def run(ref_root, script):
    cfg = os.path.join(ref_root, "config") + "/"
    out = subprocess.run([HARNESS, cfg], input=script, capture_output=True, text=True, check=True).stdout
    rows = {}
    for line in out.splitlines():
        parts = line.split()
        if not parts or parts[0] not in ("EVAL", "MOVE", "SOLVE", "BLOCK", "NIC", "NODES", "WEIGHTS", "ADD"):
            continue
        rows.setdefault(parts[0], []).append(np.array([float(x) for x in parts[1:]]))
    return rows


def system_cmd(dim, n, p, L, user_knots, sysp, time):
    uk = [] if user_knots is None else list(user_knots)
    return "SYSTEM %d %d %d %.17g %d %s %d %s %.17g\n" % (dim, n, p, L, len(uk), fmt(uk), len(sysp), fmt(sysp), time)


def lattice(n, dim, L, rng, jitter=0.1):
    """Simple-cubic start with jitter as InitCoordinateConfiguration (TDVMC.cpp:713-760)."""
    m = int(round(n ** (1.0 / dim)))
    l = L / m
    idx = np.stack(np.meshgrid(*[np.arange(m)] * dim, indexing="ij"), -1).reshape(-1, dim)[:n]
    return idx * l + (rng.uniform(size=(n, dim)) - 0.5) * l * jitter


def nic_cases(ref_root):
    """Parse the 48 known-answer displacement tests of src/test/Tests.h:76-156."""
    text = open(os.path.join(ref_root, "src", "test", "Tests.h")).read()
    body = text[text.index("void TestVectorDisplacements()"):]
    cases = []
    L = dim = None
    for line in body.splitlines():
        m = re.search(r"LBOX = (\d+);", line)
        if m:
            L = float(m.group(1))
        m = re.search(r"DIM = (\d+);", line)
        if m:
            dim = int(m.group(1))
        m = re.search(r"^\s*TestVectorDisplacement\((.*)\);", line)
        if m:
            args = [eval(a.strip(), {"sqrt": np.sqrt}) for a in m.group(1).split(",")]
            cases.append((L, dim, args))
    return cases


def k_shells(ref_root, dim, L, nshell=50):
    """The first `nshell` k shells of the reference's config/kVectors{D}D.json, scaled
    by 2 pi / L as BosonsBulk::InitSystem does (BosonsBulk.cpp:124-139)."""
    import json
    data = json.load(open(os.path.join(ref_root, "config", "kVectors%dD.json" % dim)))["data"][:nshell]
    off = np.cumsum([0] + [len(sh) for sh in data]).astype(np.int32)
    kvec = np.array([v for sh in data for v in sh], dtype=np.float64).reshape(-1, dim) * (2 * np.pi / L)
    return off, kvec


def observables(ref_root):
    """g(r) and S(k) of fixed configurations (CalculateAdditionalSystemProperties)."""
    cases = [dict(name="d1_n20", dim=1, n=20, p=10, L=20.0, knots=None, bins=50, ncfg=6, seed=41),
             dict(name="d2_n64", dim=2, n=64, p=20, L=float(np.sqrt(64 / 0.3)), knots=None, bins=64, ncfg=4,
                  seed=42),
             dict(name="d3_n343", dim=3, n=343, p=30, L=float((343 / 0.365) ** (1.0 / 3.0)), knots=None, bins=100,
                  ncfg=3, seed=43)]
    for c in cases:
        rng = np.random.default_rng(c["seed"])
        dim, n, p, L = c["dim"], c["n"], c["p"], c["L"]
        cfgs = []
        for _ in range(c["ncfg"]):
            if dim == 1:
                R = rng.uniform(-L / 2, L / 2, size=(n, dim))
            else:
                R = lattice(n, dim, L, rng, jitter=0.5) - L / 2
            # positions outside the box too: the driver does not wrap after moves
            R = R + L * rng.integers(-1, 2, size=R.shape)
            cfgs.append(R)
        cfgs = np.array(cfgs)
        script = "GRBINS %d\n" % c["bins"] + system_cmd(dim, n, p, L, c["knots"], [0.5, 1.0], 0.0)
        script += "ADDITIONAL %d\n" % len(cfgs)
        for R in cfgs:
            script += fmt(R) + "\n"
        rows = run(ref_root, script)["ADD"]
        gr, sk, kgrid = [], [], None
        for r in rows:
            ng = int(r[0])
            gr.append(r[1:1 + ng])
            ns = int(r[1 + ng])
            sk.append(r[2 + ng:2 + ng + ns])
            nk = int(r[2 + ng + ns])
            kgrid = r[3 + ng + ns:3 + ng + ns + nk]
        off, kvec = k_shells(ref_root, dim, L)
        np.savez(os.path.join(HERE, "obs_%s.npz" % c["name"]), dim=dim, n=n, p=p, L=L, gr_bins=c["bins"],
                 cfgs=cfgs, shell_off=off, kvec=kvec, ref_gr=np.array(gr), ref_sk=np.array(sk), ref_kgrid=kgrid)
        print("observables", c["name"], np.array(gr).shape, np.array(sk).shape)


# The reference's full program on a small 3D config (imaginary-time RK4, three
# written steps): its output files, as the host driver's files are compared with.
DRIVER_CONFIG = {
    "CONFIG_VERSION": "0.24", "SYSTEM_TYPE": "BosonsBulk", "OUT_DIR_SUFFIX": "", "N": 27, "LBOX": 3.6, "DIM": 3,
    "N_PARAM": 10, "RHO": 1.0, "RC": 0.0, "MC_STEP": 0.3, "MC_STEP_OFFSET": 0.0, "MC_NSTEPS": 8192,
    "MC_NTHERMSTEPS": 54, "MC_NINITIALIZATIONSTEPS": 0, "MC_VERY_FIRST_NINITIALIZATIONSTEPS": 270,
    "MC_NADDITIONALSTEPS": 0, "MC_NADDITIONALTHERMSTEPS": 0, "MC_NADDITIONALINITIALIZATIONSTEPS": 0,
    "TIMESTEP": 0.001, "TOTALTIME": 0.0025, "IMAGINARY_TIME": 1, "ODE_SOLVER_TYPE": 2,
    "LINEAR_EQUATION_SOLVER_TYPE": 0, "USE_PRECONDITIONING": 0, "USE_PARAMETER_ACCEPTANCE_CHECK": 0,
    "PARAMETER_ACCEPTANCE_CHECK_TYPE": 0, "WRITE_EVERY_NTH_STEP_TO_FILE": 1,
    "CALCULATE_ADDITIONAL_DATA_EVERY_NTH_STEP": 1000000, "WRITE_SINGLE_FILES": 0,
    "MC_NSTEP_MULTIPLICATION_FACTOR_FOR_WRITE_DATA": 1, "USE_MEAN_FOR_FINAL_PARAMETERS": 0, "USE_NORMALIZE_WF": 1,
    "USE_ADJUST_PARAMETERS": 0, "UPDATE_SAMPLES_EVERY_NTH_STEP": 0, "UPDATE_SAMPLES_PERCENT": 100.0,
    "GR_BIN_COUNT": 50, "USE_NURBS": 0, "NURBS_GRID": [0.0], "PARTICLE_TYPES": [0], "SYSTEM_PARAMS": [0.6, 1.0],
    "PARAMS_REAL": [-2.0, -2.0, -1.0, -0.5, -0.2, -0.1, -0.05, 0.0, 0.0, 0.0], "PARAMS_IMAGINARY": [0.0] * 10,
    "PARAM_PHIR": 0.0, "PARAM_PHII": 0.0,
}
# the same run with the mirrored-distance system (knots to r_max = L/2; its square well)
DRIVER_PB_CONFIG = dict(DRIVER_CONFIG, SYSTEM_TYPE="NUBosonsBulkPB", USE_NURBS=1,
                        NURBS_GRID=[round(0.2 * k, 10) for k in range(10)])
DRIVER_FILES = ("LocalEnergyR", "LocalEnergyI", "ParametersR", "ParametersI", "OtherExpectationValues",
                "LocalOperators", "timesSystem")


def driver_run(ref_root, config=DRIVER_CONFIG, name="driver_d3_n27"):
    """Runs the reference program (``ref_harness --run``) on a config (DRIVER_CONFIG,
    DRIVER_PB_CONFIG) in a scratch directory that also holds the k-vector tables it
    reads from the config's directory, and keeps the config and the output files
    above under tests/golden/<name>."""
    import json
    import shutil
    import tempfile
    dst = os.path.join(HERE, name)
    os.makedirs(dst, exist_ok=True)
    with open(os.path.join(dst, "run.config"), "w") as f:
        json.dump(config, f, indent=1)
    with tempfile.TemporaryDirectory() as tmp:
        for name in ("kVectors3D.json", "kNorm3D.csv"):
            os.symlink(os.path.join(ref_root, "config", name), os.path.join(tmp, name))
        cfg = dict(config, OUTPUT_DIRECTORY=tmp + "/out/")
        os.makedirs(cfg["OUTPUT_DIRECTORY"])
        with open(os.path.join(tmp, "run.config"), "w") as f:
            json.dump(cfg, f, indent=1)
        subprocess.run([HARNESS, "--run", os.path.join(tmp, "run.config")], check=True, capture_output=True)
        (sub,) = os.listdir(cfg["OUTPUT_DIRECTORY"])
        for name in DRIVER_FILES:
            shutil.copy(os.path.join(cfg["OUTPUT_DIRECTORY"], sub, name + ".dat"), os.path.join(dst, name + ".dat"))
    print("driver run", sub)


def pb_systems(ref_root):
    """The mirrored-distance variant (PhysicalSystems::NUBosonsBulkPB) on fixed
    configurations and single-particle moves: pb_eval_<name>.npz, the layout of
    the eval_ fixtures.  The system reads its r_max from the knot vector before
    it builds default knots, so it is always given knots (NURBS_GRID)."""
    L2 = float(np.sqrt(64 / 0.3))
    L3 = float((343 / 0.365) ** (1.0 / 3.0))
    g = np.linspace(0.0, 1.0, 20)
    knots2 = np.concatenate([[0.0], 0.7 + (L2 / 2 - 0.7) * (g[1:] - g[1]) ** 1.3 / (1 - g[1]) ** 1.3])
    systems = [
        dict(name="d3_n64_p10", dim=3, n=64, p=10, L=4.4, knots=np.linspace(0.0, 2.2, 10), sysp=[0.9, 1.0],
             ncfg=16, seed=31, jitter=0.5),
        dict(name="d2_n64_k20", dim=2, n=64, p=20, L=L2, knots=knots2, sysp=[1.0, 0.5], ncfg=16, seed=32,
             jitter=0.3),
        dict(name="d1_n20_p10", dim=1, n=20, p=10, L=20.0, knots=np.linspace(0.0, 10.0, 10), sysp=[0.5, 2.0],
             ncfg=16, seed=33),
        # the benchmark's shape: 3D N=343, rho=0.365, 30 knots on [0, L/2]
        dict(name="d3_n343_p30", dim=3, n=343, p=30, L=L3, knots=np.linspace(0.0, L3 / 2, 30), sysp=[1.0, 1.0],
             ncfg=8, seed=34, jitter=0.5),
    ]
    for sysd in systems:
        rng = np.random.default_rng(sysd["seed"])
        dim, n, p, L = sysd["dim"], sysd["n"], sysd["p"], sysd["L"]
        uR = rng.normal(0.0, 0.3, size=p)
        uI = rng.normal(0.0, 0.1, size=p)
        phiR, phiI = 0.1, -0.2
        cfgs = []
        for c in range(sysd["ncfg"]):
            if dim == 1:
                R = rng.uniform(-L / 2, L / 2, size=(n, dim))
            else:
                R = lattice(n, dim, L, rng, jitter=sysd["jitter"]) - L / 2
            cfgs.append(R)
        cfgs = np.array(cfgs)
        script = system_cmd(dim, n, p, L, sysd["knots"], sysd["sysp"], 0.0).replace("SYSTEM", "SYSTEMPB", 1)
        script += "PARAMS %s %s %.17g %.17g\n" % (fmt(uR), fmt(uI), phiR, phiI)
        script += "EVAL %d\n" % len(cfgs)
        for R in cfgs:
            script += fmt(R) + "\n"
        moves = []
        for c in range(16):
            R = cfgs[c % len(cfgs)]
            part = int(rng.integers(n))
            newpos = R[part] + rng.normal(0.0, 0.4, size=dim)
            moves.append((R, part, newpos))
        script += "MOVE %d\n" % len(moves)
        for R, part, newpos in moves:
            script += "%s %d %s\n" % (fmt(R), part, fmt(newpos))
        rows = run(ref_root, script)
        ev = np.array(rows["EVAL"])
        mv = np.array(rows["MOVE"])
        np.savez(os.path.join(HERE, "pb_eval_%s.npz" % sysd["name"]),
                 dim=dim, n=n, p=p, L=L, knots=np.asarray(sysd["knots"]), sysp=np.array(sysd["sysp"]), time=0.0,
                 uR=uR, uI=uI, phiR=phiR, phiI=phiI, cfgs=cfgs,
                 ref_lnpsi=ev[:, 0], ref_wf=ev[:, 1], ref_O=ev[:, 2:2 + p], ref_ER=ev[:, 2 + p],
                 ref_EI=ev[:, 3 + p], ref_other=ev[:, 4 + p:13 + p],
                 move_cfg=np.array([m[0] for m in moves]), move_part=np.array([m[1] for m in moves]),
                 move_new=np.array([m[2] for m in moves]), ref_move=mv)
        print("pb eval", sysd["name"], ev.shape, mv.shape)
    pb_sample(ref_root)


def pb_sample(ref_root):
    """Block averages of the reference's own Metropolis chain for the mirrored-distance
    system: the sample_d3_n27 system (3D N=27, L=3.6, square well a=0.6, b=1) with knots
    to L/2, sample_pb_d3_n27.npz (the layout of sample_d3_n27.npz plus the knots)."""
    dim, n, p, L = 3, 27, 10, 3.6
    knots = np.linspace(0.0, L / 2, p)
    rng = np.random.default_rng(35)
    uR = -0.5 * (0.6 / np.maximum(knots, 0.25)) ** 5
    uR -= uR[-1]
    uI = 0.05 * rng.normal(size=p)
    R0 = lattice(n, dim, L, rng, jitter=0.1) - L / 2
    nblock, nsamp, ntherm, step = 40, 400, n, 0.35
    script = system_cmd(dim, n, p, L, knots, [0.6, 1.0], 0.0).replace("SYSTEM", "SYSTEMPB", 1)
    script += "PARAMS %s %s 0 0\n" % (fmt(uR), fmt(uI))
    script += "SAMPLE 12346 %.17g %d %d %d %d %s\n" % (step, 50 * n, nsamp, ntherm, nblock, fmt(R0))
    blocks = np.array(run(ref_root, script)["BLOCK"])
    np.savez(os.path.join(HERE, "sample_pb_d3_n27.npz"), dim=dim, n=n, p=p, L=L, sysp=np.array([0.6, 1.0]),
             knots=knots, uR=uR, uI=uI, R0=R0, nblock=nblock, nsamp=nsamp, ntherm=ntherm, step=step, blocks=blocks)
    print("pb sample blocks", blocks.shape)


def main():
    ref_root = (sys.argv[1] if len(sys.argv) > 1 and sys.argv[1] not in ("obs", "driver", "pb", "driver-pb")
                else "/root/reference")
    if not os.path.exists(HARNESS):
        subprocess.check_call([os.path.join(ROOT, "oracle", "ref", "build_ref.sh"), ref_root])
    if "obs" in sys.argv[1:]:
        observables(ref_root)
        return
    if "driver" in sys.argv[1:]:
        driver_run(ref_root)
        return
    if "driver-pb" in sys.argv[1:]:
        driver_run(ref_root, DRIVER_PB_CONFIG, "driver_pb_d3_n27")
        return
    if "pb" in sys.argv[1:]:
        pb_systems(ref_root)
        return
    driver_run(ref_root)
    driver_run(ref_root, DRIVER_PB_CONFIG, "driver_pb_d3_n27")
    pb_systems(ref_root)
    observables(ref_root)

    # ---- NIC known answers (the reference's own unit test vectors) ----
    cases = nic_cases(ref_root)
    script = ""
    ins, exp = [], []
    for L, dim, args in cases:
        k = 3 if dim == 3 else 1
        ri, rj = args[:k], args[k:2 * k]
        script += "NIC %d %.17g 1 %s %s\n" % (k, L, fmt(ri), fmt(rj))
        pad = lambda v: list(v) + [0.0] * (3 - len(v))
        ins.append([L, k] + pad(ri) + pad(rj))
        exp.append([args[2 * k]] + pad(args[2 * k + 1:]))
    rows = run(ref_root, script)["NIC"]
    refout = np.array([list(r) + [0.0] * (4 - len(r)) for r in rows])
    np.savez(os.path.join(HERE, "nic_kat.npz"), inputs=np.array(ins), expected=np.array(exp), reference=refout)
    print("nic cases", len(cases))

    # ---- systems for fixed-configuration evaluation ----
    systems = []
    # 1D, N=20, L=20, P=10 uniform, square well (BosonsBulk.cpp:268-271)
    systems.append(dict(name="d1_n20_p10", dim=1, n=20, p=10, L=20.0, knots=None, sysp=[0.5, 2.0], time=0.0,
                        ncfg=24, seed=11))
    # same with the quench rule active (BosonsBulk.cpp:239-242)
    systems.append(dict(name="d1_n20_p10_quench", dim=1, n=20, p=10, L=20.0, knots=None,
                        sysp=[0.5, 2.0, 0.5, 0.8, 4.0], time=1.0, ncfg=8, seed=12))
    # 2D, N=64, density 0.3, 20 non-uniform knots through SetNodes (BosonsBulk.cpp:35-44)
    L2 = float(np.sqrt(64 / 0.3))
    g = np.linspace(0.0, 1.0, 20)
    knots2 = np.concatenate([[0.0], 0.7 + (L2 / 2 - 0.7) * (g[1:] - g[1]) ** 1.3 / (1 - g[1]) ** 1.3])
    # (the parity set of the 2D Lennard-Jones configuration: 256 configurations on
    # the 8x8 lattice with 0.05 jitter, seed 7)
    systems.append(dict(name="d2_n64_k20", dim=2, n=64, p=20, L=L2, knots=knots2, sysp=[1.0, 0.5], time=0.0,
                        ncfg=256, seed=7, jitter=0.05))
    # 3D, N=64, L=4 (the fixture box of src/VMCSampler.h:18)
    systems.append(dict(name="d3_n64_p10", dim=3, n=64, p=10, L=4.0, knots=None, sysp=[0.6, 1.0], time=0.0,
                        ncfg=16, seed=14))
    # 3D, N=343, density 0.365, 30 parameters (the benchmark system)
    L3 = float((343 / 0.365) ** (1.0 / 3.0))
    systems.append(dict(name="d3_n343_p30", dim=3, n=343, p=30, L=L3, knots=None, sysp=[0.9, 1.0], time=0.0,
                        ncfg=32, seed=15))

    for sysd in systems:
        rng = np.random.default_rng(sysd["seed"])
        dim, n, p, L = sysd["dim"], sysd["n"], sysd["p"], sysd["L"]
        uR = rng.normal(0.0, 0.3, size=p)
        uI = rng.normal(0.0, 0.1, size=p)
        phiR, phiI = 0.1, -0.2
        cfgs = []
        for c in range(sysd["ncfg"]):
            if dim == 1:
                R = rng.uniform(-L / 2, L / 2, size=(n, dim))
            else:
                R = lattice(n, dim, L, rng, jitter=sysd.get("jitter", 0.5)) - L / 2
            cfgs.append(R)
        cfgs = np.array(cfgs)
        script = system_cmd(dim, n, p, L, sysd["knots"], sysd["sysp"], sysd["time"])
        script += "PARAMS %s %s %.17g %.17g\n" % (fmt(uR), fmt(uI), phiR, phiI)
        script += "WEIGHTS\n"
        script += "EVAL %d\n" % len(cfgs)
        for R in cfgs:
            script += fmt(R) + "\n"
        # single-particle moves on the first configurations
        moves = []
        nmove = 16
        for c in range(nmove):
            R = cfgs[c % len(cfgs)]
            part = int(rng.integers(n))
            newpos = R[part] + rng.normal(0.0, 0.4, size=dim)
            moves.append((R, part, newpos))
        script += "MOVE %d\n" % nmove
        for R, part, newpos in moves:
            script += "%s %d %s\n" % (fmt(R), part, fmt(newpos))
        rows = run(ref_root, script)
        ev = np.array(rows["EVAL"])
        mv = np.array(rows["MOVE"])
        np.savez(os.path.join(HERE, "eval_%s.npz" % sysd["name"]),
                 dim=dim, n=n, p=p, L=L, knots=np.zeros(0) if sysd["knots"] is None else sysd["knots"],
                 sysp=np.array(sysd["sysp"]), time=sysd["time"], uR=uR, uI=uI, phiR=phiR, phiI=phiI,
                 cfgs=cfgs, ref_nodes=rows["NODES"][0][1:], ref_weights=rows["WEIGHTS"][0][1:],
                 ref_lnpsi=ev[:, 0], ref_wf=ev[:, 1], ref_O=ev[:, 2:2 + p], ref_ER=ev[:, 2 + p],
                 ref_EI=ev[:, 3 + p], ref_other=ev[:, 4 + p:13 + p], ref_lj=ev[:, 13 + p],
                 move_cfg=np.array([m[0] for m in moves]), move_part=np.array([m[1] for m in moves]),
                 move_new=np.array([m[2] for m in moves]), ref_move=mv)
        print("eval", sysd["name"], ev.shape, mv.shape)

    # ---- TDVP linear solve (SolveForParametersDot, TDVMC.cpp:1713-1828) ----
    solve_rows = []
    for p, seed in ((10, 21), (30, 22)):
        rng = np.random.default_rng(seed)
        nsamp = 4 * p
        O = rng.normal(size=(nsamp, p)) @ rng.normal(size=(p, p)) * 0.3 + rng.normal(size=p) * 2.0
        ER = rng.normal(size=nsamp) * 0.5 - 3.0 + O[:, 0] * 0.1
        EI = rng.normal(size=nsamp) * 0.2 + O[:, 1] * 0.05
        mom = dict(O=O.mean(0), ER=ER.mean(), EI=EI.mean(), OO=O.T @ O / nsamp,
                   OER=(O * ER[:, None]).mean(0), OEI=(O * EI[:, None]).mean(0))
        script = system_cmd(3, 8, p, 4.0, None, [0.5, 1.0], 0.0)
        combos = [(imag, pre, solver) for imag in (0, 1) for pre in (0, 1) for solver in (0, 1)]
        for imag, pre, solver in combos:
            script += "SOLVE %d %d %d %s %.17g %.17g %s %s %s\n" % (imag, pre, solver, fmt(mom["O"]), mom["ER"],
                                                                 mom["EI"], fmt(mom["OO"]), fmt(mom["OER"]),
                                                                 fmt(mom["OEI"]))
        rows = run(ref_root, script)["SOLVE"]
        for (imag, pre, solver), r in zip(combos, rows):
            solve_rows.append(dict(p=p, imag=imag, pre=pre, solver=solver, mom=mom, out=r))
    np.savez(os.path.join(HERE, "solve.npz"),
             p=np.array([r["p"] for r in solve_rows]), imag=np.array([r["imag"] for r in solve_rows]),
             pre=np.array([r["pre"] for r in solve_rows]), solver=np.array([r["solver"] for r in solve_rows]),
             **{"O_%d" % i: r["mom"]["O"] for i, r in enumerate(solve_rows)},
             **{"ER_%d" % i: r["mom"]["ER"] for i, r in enumerate(solve_rows)},
             **{"EI_%d" % i: r["mom"]["EI"] for i, r in enumerate(solve_rows)},
             **{"OO_%d" % i: r["mom"]["OO"] for i, r in enumerate(solve_rows)},
             **{"OER_%d" % i: r["mom"]["OER"] for i, r in enumerate(solve_rows)},
             **{"OEI_%d" % i: r["mom"]["OEI"] for i, r in enumerate(solve_rows)},
             **{"out_%d" % i: r["out"] for i, r in enumerate(solve_rows)})
    print("solve cases", len(solve_rows))

    # ---- sampled averages from the reference's own Metropolis chain ----
    # 3D, N=27, L=3.6, square well; block averages give the 3-sigma band.
    dim, n, p, L = 3, 27, 10, 3.6
    rng = np.random.default_rng(31)
    r_greville = np.linspace(0.0, L / 2, p)
    uR = -0.5 * (0.6 / np.maximum(r_greville, 0.25)) ** 5  # McMillan-like ramp
    uR -= uR[-1]
    uI = 0.05 * rng.normal(size=p)
    R0 = lattice(n, dim, L, rng, jitter=0.1) - L / 2
    nblock, nsamp, ntherm, step = 40, 400, n, 0.35
    script = system_cmd(dim, n, p, L, None, [0.6, 1.0], 0.0)
    script += "PARAMS %s %s 0 0\n" % (fmt(uR), fmt(uI))
    script += "SAMPLE 12345 %.17g %d %d %d %d %s\n" % (step, 50 * n, nsamp, ntherm, nblock, fmt(R0))
    blocks = np.array(run(ref_root, script)["BLOCK"])
    np.savez(os.path.join(HERE, "sample_d3_n27.npz"), dim=dim, n=n, p=p, L=L, sysp=np.array([0.6, 1.0]),
             uR=uR, uI=uI, R0=R0, nblock=nblock, nsamp=nsamp, ntherm=ntherm, step=step, blocks=blocks)
    print("sample blocks", blocks.shape)


if __name__ == "__main__":
    main()
