"""Builds tests/emulation/_build/libant_emu.so: the ant kernel's body, taken
from gplsaco_gb300/csrc/faco_kernels.cu as it is, compiled for the host with
the warp shim (warp_shim.h), plus a C entry (emulator_entry.cpp) that runs one
engine-mode ant with 32 lane threads.  The only edits are mechanical: the
kernel signature, thread/block indices (one warp, one block), the
sqrt.approx estimate of the integer EUC_2D length (std::sqrt: the exact
integer correction that follows it decides the result either way), and a
uniformity check after every construction step.  Test infrastructure only.

    python tests/emulation/make_emulator.py
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
CSRC = ROOT / "gplsaco_gb300" / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libant_emu.so"


def generate() -> Path:
    BUILD.mkdir(exist_ok=True)
    common = (CSRC / "faco_common.cuh").read_text()
    common = common.replace("#include <cuda_runtime.h>", '#include "warp_shim.h"')
    common = common.replace('    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));', "    r = std::sqrt(x);")
    (BUILD / "faco_common.cuh").write_text(common)
    (BUILD / "faco_ant.cuh").write_text((CSRC / "faco_ant.cuh").read_text())
    src = (CSRC / "faco_kernels.cu").read_text()
    body = src[src.index("__device__ __forceinline__ void load_parent("):src.index("namespace {\n// The dynamic shared")]
    signature = ("template <int MODE>\n__global__ void __launch_bounds__(kMaxWarpsPerBlock * 32, "
                 "kAntBlocksPerSM) ant_kernel(const AntLaunch L) {")
    if signature not in body:
        raise SystemExit("kernel source changed: cannot find the ant kernel's signature")
    body = body.replace(signature, "template <int MODE>\nvoid ant_kernel_emu(const AntLaunch L, unsigned char* smem) {")
    body = body.replace("    extern __shared__ __align__(16) unsigned char smem[];\n", "")
    body = body.replace("threadIdx.x", "tl_lane").replace("blockIdx.x", "0u").replace("blockDim.x", "32u")
    body = body.replace("__syncthreads()", "__syncwarp()")
    check = ('uniform_check("{0}", current, r.steps, r.mne, cost, run.m, run.p, run.t, (unsigned)run.dir, '
             'q.pending, q.tail);')
    for old, new in (("                follow = full;\n                if (f) continue;",
                      "                follow = full;\n                " + check.format("batched") +
                      "\n                if (f) continue;"),
                     ("            current = selected;\n            __syncwarp();\n        }",
                      "            current = selected;\n            __syncwarp();\n            " +
                      check.format("single") + "\n        }")):
        if old not in body:
            raise SystemExit(f"kernel source changed: cannot place the uniformity check ({old[:40]!r})")
        body = body.replace(old, new)
    head = ('#include <thread>\n#include <vector>\n#include "faco_ant.cuh"\n#include "uniform_check.h"\n'
            "std::mutex g_atomic;\nthread_local Warp* tl_warp = nullptr;\nthread_local unsigned tl_lane = 0;\n"
            "namespace faco {\n"
            "__device__ inline std::uint32_t list_start(unsigned long long, std::uint32_t, std::uint32_t, "
            "const node_t*, std::uint32_t) { return 0; }\n"
            "struct RefControl { const node_t* start_nodes; std::uint32_t start_count; };\n")
    out = BUILD / "emu.cpp"
    out.write_text(head + body + "}  // namespace faco\n" + (HERE / "emulator_entry.cpp").read_text())
    return out


def build(force: bool = False) -> Path:
    sources = [HERE / "warp_shim.h", HERE / "uniform_check.h", HERE / "emulator_entry.cpp", Path(__file__),
               CSRC / "faco_common.cuh", CSRC / "faco_ant.cuh", CSRC / "faco_kernels.cu"]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in sources):
        return LIB
    cpp = generate()
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wno-unknown-pragmas",
                    f"-I{BUILD}", f"-I{HERE}", str(cpp), "-o", str(tmp), "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
