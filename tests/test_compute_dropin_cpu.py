"""The drop-in compute() runs: the reference's own host program (main,
initParameters, read_PDB, the updater hooks; its .cpp files compiled where
they lie) with mt_gb300/host/mtg_compute.cpp in place of its CUDA sources,
linked against a recording stand-in of the engine's C ABI
(tests/dropin/mtg_recorder.cpp) instead of libmtg.so, so it runs on a CPU.
The run has pair-list rebuilds, hydrolysis, stride output with energies and
forces, tubule length with barriers and constant concentration on.  The
recorded sequence of engine calls and updater hooks is compared step by step
with the order of the reference's step loop (src/compute_cuda.cu:1137-1238),
restated below.  Needs the reference tree; skipped where it is absent."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "mt_gb300", "host")
WRAPPED = ("_Z9hydrolysev", "_Z6updatexPi", "_Z9mt_lengthxPi", "_Z11change_concPiS_")

CONFIG = """device 0
rseed 1234567
dt 200
LJPairsCutoff 8
LJPairsUpdateFreq 10
stride 20
steps 100
forcefield ff.conf
conditions cond.conf
coordinates_xyz xyz.pdb
coordinates_ang ang.pdb
restart_xyz restart/xyz_<run>.xyz
restart_ang restart/ang_<run>.xyz
restartkey restart/key.txt
dcd_xyz dcd/out_<run>.dcd
dcd_ang dcd/out_<run>.dcd_ang
fix 1
runnum 2
is_assembly yes
tubule_length yes
output_energy yes
output_force yes
"""
COND = """Temp 300
viscosity 2.85e4
is_const_conc yes
conc 10
hydrolysis yes
khydro 4000000
freeze_temp 1.0
alpha 5.0
"""
PAR = dict(steps=100, stride=20, freq=10, hydrostep=25, lj_on=1, is_assembly=1, hydrolysis=1, out_energy=1,
           out_force=1, tub_length=1, barrier=1, const_conc=1)


def reference_order(par, change_conc_returns):
    """Engine work and host hooks of the reference's step loop, in order
    (src/compute_cuda.cu:1137-1238), named by the engine call that replaces
    each kernel launch or copy.  change_conc's return values are taken from
    the run: they decide whether the extra flags and the state go back to
    the device (:1195-1206)."""
    ev, rets = [], iter(change_conc_returns)
    for s in range(par["steps"]):
        if s % par["freq"] == 0 and (par["lj_on"] or par["is_assembly"]):        # :1140-1151
            ev.append(("rebuild", s))
        if par["hydrolysis"] and s % par["hydrostep"] == 0 and s != 0:          # :1153-1160
            ev += [("hydrolyse", s), ("set_gtp", s)]
        if s % par["stride"] == 0:                                               # :1163
            if par["out_energy"]:                                                # :1165-1170
                ev.append(("energies", s))
            ev.append(("download_state", s))                                     # :1172-1178 (f, r)
            if par["tub_length"]:                                                # :1181
                if s != 0:
                    ev.append(("mt_length", s))                                  # :1186-1187
                    if par["barrier"]:
                        ev.append(("set_on_tubule", s))                          # :1189-1193
                    if par["const_conc"]:
                        r = next(rets)
                        ev.append(("change_conc", s, r))                         # :1195-1201
                        if r:
                            ev += [("set_extra", s), ("upload_state", s)]        # :1202-1205
                    ev.append(("update", s))                                     # :1214
                else:
                    ev += [("update", s), ("mt_length", s)]                      # :1217-1218
            else:
                ev.append(("update", s))                                         # :1223
        ev.append(("step", s))                                                   # :1228-1237
    return ev


def recorded_order(lines):
    """The run's MTG/HOOK lines as (event, step[, value]); host calls belong
    to the step that runs next."""
    ev, cur, body = [], 0, False
    for ln in lines:
        m = re.match(r"(MTG|HOOK) (\w+)(.*)", ln)
        if not m:
            continue
        kind, name, rest = m.group(1), m.group(2), m.group(3)
        if name == "create":
            continue
        if name == "upload_state" and not body:
            continue                                  # the initial upload (initIntegration)
        body = True
        if name == "destroy" or name == "step_call":
            continue
        if name == "device_step":
            s = int(re.search(r"step=(\d+)", rest).group(1))
            ev.append(("step", s))
            cur = s + 1
        elif name in ("device_rebuild", "rebuild_pairs"):
            ev.append(("rebuild", cur))
        elif name == "change_conc":
            ev.append(("change_conc", cur, int(re.search(r"ret=(-?\d+)", rest).group(1))))
        elif name in ("mt_length", "update"):
            s = int(re.search(r"step=(\d+)", rest).group(1))
            assert s == cur, (ln, cur)
            ev.append((name, s))
        else:
            ev.append((name, cur))
    return ev


@pytest.fixture(scope="module")
def dropin_run(tmp_path_factory):
    from oracle.reftree import reference_tree
    ref = reference_tree()
    if not ref:
        pytest.skip("reference sources absent")
    r = subprocess.run(["make", "-s", "-C", HOST, "objs", f"REF={ref}"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    tmp = tmp_path_factory.mktemp("dropin")
    objs = [os.path.join(HOST, "_build", f"{n}.o") for n in
            ("main", "preparator", "updater", "configreader", "pdbio", "dcdio", "xyzio", "wrapper", "timer",
             "parameters", "globals", "mtg_compute")]
    exe = str(tmp / "mt_rec")
    wrap = ",".join(f"--wrap={w}" for w in WRAPPED)
    r = subprocess.run(["g++", "-O1", "-std=c++14", "-I", os.path.join(ROOT, "include"), "-o", exe, *objs,
                        os.path.join(ROOT, "tests", "dropin", "mtg_recorder.cpp"), f"-Wl,{wrap}"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    cc = os.path.join(ref, "initial", "constconc", "10")
    shutil.copy(os.path.join(cc, "xyz_10.pdb"), tmp / "xyz.pdb")    # 13 PF lattice + chain-X extra dimers
    shutil.copy(os.path.join(cc, "ang_10.pdb"), tmp / "ang.pdb")
    shutil.copy(os.path.join(ref, "template", "morse.conf"), tmp / "ff.conf")
    (tmp / "config.conf").write_text(CONFIG)
    (tmp / "cond.conf").write_text(COND)
    for d in ("dcd", "restart"):
        (tmp / d).mkdir()
    r = subprocess.run([exe, "config.conf"], cwd=tmp, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-2000:])
    return r.stdout.splitlines(), tmp


def test_dropin_call_sequence_matches_reference_loop(dropin_run):
    lines, _ = dropin_run
    got = recorded_order(lines)
    rets = [e[2] for e in got if e[0] == "change_conc"]
    assert any(rets), "constant concentration never re-inserted a dimer: the branch is untested"
    want = reference_order(PAR, rets)
    for k, (a, b) in enumerate(zip(got, want)):
        assert a == b, f"event {k}: drop-in {a}, reference order {b}\n{got[max(0, k - 5):k + 5]}"
    assert len(got) == len(want), (len(got), len(want))


def test_dropin_maps_parameters_and_topology(dropin_run):
    """mtg_create receives the reference's Parameters/Topology field by field
    (to_mtg in mtg_compute.cpp) as initParameters and read_PDB set them."""
    lines, _ = dropin_run
    cr = next(ln for ln in lines if ln.startswith("MTG create "))
    kv = dict(x.split("=") for x in cr.split()[2:])
    assert (kv["Ntot"], kv["Ntr"], kv["maxH"]) == ("286", "2", "1")
    # list capacities: AssemblyInit (src/preparator.cpp:721-722) and LJ (src/compute_cuda.cu:1076)
    assert (kv["maxLong"], kv["maxLat"], kv["maxLJ"]) == ("8", "16", "256")
    assert kv["extra"] == str(2 * 234)                     # chain X in both trajectories
    assert float(kv["dt"]) == 200 and float(kv["Temp"]) == 300 and float(kv["viscosity"]) == 2.85e4
    assert int(kv["ljpairsupdatefreq"]) == 10 and float(kv["ljpairscutoff"]) == 8
    assert kv["is_assembly"] == "1" and kv["hdi_on"] == "0" and kv["barrier"] == "1" and kv["lj_on"] == "1"
    assert int(kv["rseed"]) == 1234567 and float(kv["zs0"]) == 160.0     # rep_h of the force field
    # derived constants as src/preparator.cpp:209-219 computes them
    import math
    assert abs(float(kv["gammaR"]) - 6 * math.pi * 2.85e4 * 2.0) / float(kv["gammaR"]) < 1e-5
    assert abs(float(kv["gammaTheta"]) - 8 * math.pi * 2.85e4 * 8.0) / float(kv["gammaTheta"]) < 1e-5


def test_dropin_outputs_written(dropin_run):
    """The reference's own writers ran from the drop-in's host state: one DCD
    frame per stride step per trajectory and the final PDBs."""
    _, tmp = dropin_run
    for t in range(2):
        for suffix in (".dcd", ".dcd_ang"):
            f = tmp / "dcd" / f"out_{t}{suffix}"
            assert f.exists() and f.stat().st_size > 0
    assert (tmp / "result_xyz.pdb").exists() and (tmp / "result_ang.pdb").exists()
