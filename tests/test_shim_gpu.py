"""The reference-side binding (include/gbsa_shim.hpp) against the reference's own CPU
code (GB300 only).

oracle/shim_check (built by oracle/build_ref.sh from the reference's sources and linked
with libgbsa.so) populates a StrobemerIndex on the GPU through gbsa_shim::gpu_populate,
then for every read compares the reference's find_nams / find_nams_rescue, run on the
host vectors the shim filled, with gbsa_shim::find_nams / find_nams_rescue on the GPU
index (half the reads starting from a one-record NAM buffer, so the shim's retry on
GBSA_ERR_CAPACITY runs).
"""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from gpu_index_test_gb300 import synth

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(REPO, "oracle", "_ref", "shim_check")


def test_shim_matches_the_reference_find_nams():
    if not os.path.exists(SHIM):
        pytest.skip("oracle/_ref/shim_check not built: the reference's sources are not on this host")
    g = synth.make_genome(synth.genome_params("C2", scale=0.004, seed=131))   # 400 kbp, duplications + STRs
    reads = synth.make_reads(g, synth.read_params("C2", n_units=1500, seed=132))
    with tempfile.TemporaryDirectory() as d:
        case = os.path.join(d, "case.bin")
        with open(case, "wb") as f:
            np.array([len(g.lengths)], np.uint32).tofile(f)
            g.lengths.astype(np.uint64).tofile(f)
            g.seq.tofile(f)
            np.array([reads.n], np.uint32).tofile(f)
            reads.lengths.astype(np.uint32).tofile(f)
            reads.seq.tofile(f)
        r = subprocess.run([SHIM, case], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert line, r.stderr[-2000:]
    res = json.loads(line[-1])
    assert res["reads"] == reads.n and res["nams"] > 0
    assert res["find_nams_mismatches"] == 0 and res["fraction_mismatches"] == 0 and res["rescue_mismatches"] == 0
    assert res["capacity_retries"] > 0
    assert r.returncode == 0
