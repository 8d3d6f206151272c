"""Location of the reference source tree (klyshko/MT), for the recipes that
compile parts of it as test infrastructure (oracle/Makefile `ref`,
mt_gb300/host/Makefile).  Taken from the MTG_REFERENCE_TREE environment
variable, else a checkout named ``reference`` beside this repository; None
when neither holds the reference's src/ directory (the GPU host, for one)."""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_tree():
    for cand in (os.environ.get("MTG_REFERENCE_TREE"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isfile(os.path.join(cand, "src", "compute_cuda.cu")):
            return os.path.abspath(cand)
    return None
