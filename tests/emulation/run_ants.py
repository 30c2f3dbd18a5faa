"""Runs engine-mode ants of the emulated ant kernel (make_emulator.py)
against the oracle's ant with the same Philox draws; exits non-zero on the
first difference.  A warp race or an intrinsic reached by some lanes only
aborts the emulation itself.  Test infrastructure only.

    python tests/emulation/run_ants.py KIND N K ITERATIONS [MODE:LS,...]

The optional last argument limits the run to those (kernel variant, LS
mode) pairs, e.g. 4:0,6:0.
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE))

import make_emulator  # noqa: E402
from gplsaco_gb300 import instances  # noqa: E402
from oracle import oracle  # noqa: E402

def _state(xy, k, b, w, iterations, seed):
    prep = oracle.prepare(xy, k, b, w)
    key = oracle.lib().orc_colony_key(seed, 1)
    if iterations:
        res = oracle.run_colony(xy, prep, ants=16, k=k, b=b, w=w, mne=8, iterations=iterations, key=key,
                                want_trace=False)
        return prep, key, res["tour"].astype(np.uint32), np.ascontiguousarray(res["products"], np.float32)
    return prep, key, prep["initial"].astype(np.uint32), oracle.heuristic(xy, prep["primary"]) * np.float32(1e-6)


def _ant(emu, mode, ls_mode, xy, prep, key, parent, products, k, b, w, batch, ant):
    n = len(xy)
    m = oracle.euc2d_matrix(xy)
    pos = np.empty(n, np.int64)
    pos[parent] = np.arange(n)
    nbr = (parent[(pos + 1) % n] | (parent[(pos - 1) % n] << 16)).astype(np.uint32)
    arrays = dict(xy=np.ascontiguousarray(xy, np.int32), primary=np.ascontiguousarray(prep["primary"], np.uint16),
                  backup=np.ascontiguousarray(prep["backup"] if b else np.zeros((n, 1)), np.uint16),
                  ls=np.ascontiguousarray(prep["ls"], np.uint16),
                  ls_dist=np.ascontiguousarray(m[np.arange(n)[:, None], prep["ls"].astype(np.int64)], np.int32),
                  parent=np.ascontiguousarray(parent, np.uint16))
    tour, costs, counts, err = np.zeros(n, np.uint16), np.zeros(2, np.int64), np.zeros(3, np.uint32), np.zeros(1, np.uint32)
    cost = int(np.sum(m[parent, np.roll(parent, -1)]))
    rc = emu.emu_ant(mode, n, k, b, w, *(arrays[x].ctypes.data for x in ("xy", "primary", "backup", "ls",
                                                                          "ls_dist", "parent")),
                     nbr.ctypes.data, products.ctypes.data, key, batch, ant, 8, cost, ls_mode, tour.ctypes.data,
                     costs.ctypes.data, counts.ctypes.data, err.ctypes.data)
    assert rc == 0, mode
    uni = np.array([0.0] + [oracle.lib().orc_uniform(key, batch, ant, s) for s in range(1, n)])
    ref = oracle.ant(parent, prep["ls"], 8, 100000, xy=xy, uniforms=uni,
                     start=oracle.lib().orc_start_node(key, batch, ant, n), primary=prep["primary"],
                     products32=products, backup=prep["backup"] if b else None, ls_mode=ls_mode)
    ctx = (mode, ls_mode, batch, ant)
    assert err[0] == 0, ctx
    assert np.array_equal(tour.astype(np.uint32), ref["tour"]), ctx
    assert (int(costs[0]), int(costs[1])) == (ref["construction_cost"], ref["final_cost"]), ctx
    assert int(counts[0]) == ref["steps"], ctx
    return int(counts[0])



# (kernel variant, LS mode): steps one at a time (0), in batches (5), the
# batched build for full panels (7), the global-workspace variants (4, 6),
# and the 2-opt + Or-opt local search; the first three with every ant
ANTS = ((3, 0), (3, 1), (7, 2), (11, 5))
MAIN_VARIANTS = ((0, 0), (5, 0), (7, 0))
VARIANTS = MAIN_VARIANTS + ((4, 0), (6, 0), (0, 1), (6, 1))


def main() -> None:
    kind, n, k, iterations = sys.argv[1], int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4])
    emu = C.CDLL(str(make_emulator.build()))
    vp = C.c_void_p
    emu.emu_ant.argtypes = [C.c_uint32] * 5 + [vp] * 8 + [C.c_ulonglong, C.c_uint32, C.c_uint32, C.c_uint32,
                                                        C.c_longlong, C.c_uint32, vp, vp, vp, vp]
    xy = instances.uniform(n, 500 + n) if kind == "uniform" else instances.clustered(n, 500 + n)
    b, w = min(64, n - 1 - k), min(20, n - 1)
    prep, key, parent, products = _state(xy, k, b, w, iterations, seed=3)
    variants = VARIANTS
    if len(sys.argv) > 5:
        variants = tuple(tuple(int(x) for x in v.split(":")) for v in sys.argv[5].split(","))
    steps = runs = 0
    for mode, ls_mode in variants:
        ants = ANTS if (mode, ls_mode) in MAIN_VARIANTS else ANTS[::2]
        for batch, ant in ants:
            steps += _ant(emu, mode, ls_mode, xy, prep, key, parent, products, k, b, w, batch, ant)
            runs += 1
    assert steps > 0
    print(f"{kind} n={n} k={k} it={iterations}: {runs} ants over {len(variants)} variants equal the oracle "
          f"({steps} construction steps)")


if __name__ == "__main__":
    main()
