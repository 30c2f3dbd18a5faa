"""The ant kernel's own source run on the CPU (tests/emulation): engine-mode
ants -- steps taken one at a time (ant_kernel<0>) and parent-following steps
taken in batches (ant_kernel<5>, and ant_kernel<7>, the build of the same
steps for panels beyond one wave), the global-memory-workspace variants
(ant_kernel<4>, <6>) and the 2-opt + Or-opt local search -- against the
oracle's ant with the same Philox draws, bit for bit: final tour,
construction and final lengths, step count.  The warp intrinsics are emulated with 32 threads that are delayed at
random before every barrier, and the lanes' per-ant registers are compared
after every step, so a warp race (lanes that read shared state while another
lane writes it) fails the run instead of hiding behind lockstep execution.
Each case runs in a child process (tests/emulation/run_ants.py).

States: the prepared tour with plain heuristics (early walks) and an oracle
colony after 100-150 iterations (converged trails: long walks along the
parent tour, where the batches carry most steps)."""
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


# the last case is above 2048 nodes, where every relocation is deferred into
# a run, with the variants the engine runs there (global-memory workspace)
# and the shared-memory one
@pytest.mark.parametrize("kind,n,k,iterations,variants", [("uniform", 60, 8, 0, None),
                                                           ("clustered", 300, 20, 100, None),
                                                           ("uniform", 800, 16, 150, None),
                                                           ("clustered", 2500, 16, 20, "4:0,6:0,0:0")])
def test_emulated_kernel_ants_match_oracle(oracle, kind, n, k, iterations, variants):
    args = [kind, str(n), str(k), str(iterations)] + ([variants] if variants else [])
    out = subprocess.run([sys.executable, str(ROOT / "tests" / "emulation" / "run_ants.py")] + args,
                         capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, (out.stdout[-2000:], out.stderr[-3000:])
    assert "equal the oracle" in out.stdout
