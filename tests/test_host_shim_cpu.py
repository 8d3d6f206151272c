"""The drop-in boundary links: the reference's own host program (its .cpp
files compiled where they lie, main() at src/main.cpp:19) together with
mt_gb300/host/mtg_compute.cpp, which implements the reference's
compute(Coord*, Coord*, Parameters&, Topology&, Energies*)
(src/compute_cuda.cuh:17) on top of libmtg.so.  Building needs the
reference tree; the test is skipped where it is absent."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "mt_gb300", "host")


def test_reference_program_links_against_the_engine(engine_mod):
    from oracle.reftree import reference_tree
    ref = reference_tree()
    if not ref:
        pytest.skip("reference sources absent")
    r = subprocess.run(["make", "-s", "-C", HOST, f"REF={ref}"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = os.path.join(HOST, "_build", "mt")
    dyn = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True, check=True).stdout
    assert "libmtg.so" in dyn
    # compute() comes from the shim, the rest of the program from the reference
    syms = subprocess.run(["nm", "-C", os.path.join(HOST, "_build", "mtg_compute.o")], capture_output=True,
                          text=True, check=True).stdout
    assert re.search(r" T compute\(Coord\*, Coord\*, Parameters&, Topology&, Energies\*\)", syms), syms
    used = set(re.findall(r" U (mtg_\w+)", syms))
    exported = set(re.findall(r"\b(mtg_\w+)\b", subprocess.run(
        ["nm", "-D", "--defined-only", engine_mod.LIB_PATH], capture_output=True, text=True, check=True).stdout))
    assert used and used <= exported, used - exported
