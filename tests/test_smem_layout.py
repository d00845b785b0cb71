"""Shared-memory budget of every render_kernel instantiation, checked on the host.

The kernels' speed depends on how many blocks share an SM and on how much of the SM's 256 KB of
shared memory plus L1 is left to L1.  A host-only program compiled against render_core.cuh prints,
for each instantiation, the dynamic shared memory per block (warp_smem_floats of its SmemLayout,
times the block's warps) and the blocks per SM its __launch_bounds__ asks for.  The test holds:
  * every instantiation: its blocks fit the 228 KB an SM offers (each block also reserves 1 KB);
  * the forward kernels (six blocks; five for the MSI background's and the batch launch's): their
    blocks fit the 196 KB carve-out, which leaves 60 KB of L1 for the link and density gathers.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

SM_SHARED = 228 * 1024        # shared memory an SM can give its blocks
BLOCK_RESERVED = 1024         # per block, reserved by the system
FORWARD_CARVEOUT = 196 * 1024

SOURCE = r"""
#include "render_core.cuh"
#include <cstdio>
using namespace svx::rk;
template <typename ShT, int MODE, bool MULTI, bool BG>
void row(const char* dt, int cap) {
  constexpr bool five = MULTI || BG;
  const int scap = (MODE == kFusedFwd || MODE == kFusedRev) ? 0 : cap;
  const size_t b = sizeof(float) * (size_t)warp_smem_floats(smem_layout<ShT, MODE, five>(27, scap)) * kWarps;
  printf("%s %d %d %d %d %zu %d\n", dt, MODE, (int)MULTI, (int)BG, scap, b, blocks_per_sm_bound(MODE, MULTI, BG));
}
template <typename ShT>
void all(const char* dt) {
  row<ShT, kFwd, false, false>(dt, 0);
  row<ShT, kFwd, true, false>(dt, 0);
  row<ShT, kFwd, false, true>(dt, 0);
  row<ShT, kFusedFwd, false, false>(dt, 0);
  row<ShT, kFusedFwd, true, false>(dt, 0);
  row<ShT, kFusedFwd, false, true>(dt, 0);
  row<ShT, kFusedRev, false, false>(dt, 0);
  row<ShT, kFusedRev, true, false>(dt, 0);
  for (int cap : {0, 48}) {
    row<ShT, kFused, false, false>(dt, cap);
    row<ShT, kFused, true, false>(dt, cap);
    row<ShT, kFused, false, true>(dt, cap);
    row<ShT, kBwd, false, false>(dt, cap);
    row<ShT, kBwd, false, true>(dt, cap);
  }
}
int main() {
  all<float>("f32");
  all<__nv_bfloat16>("bf16");
  all<__half>("f16");
  return 0;
}
"""


@pytest.fixture(scope="module")
def layout_rows(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("smem")
    src, exe = d / "layout.cu", d / "layout"
    src.write_text(SOURCE)
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}",
           f"-I{ROOT / 'svox2_gb300' / 'csrc'}", str(src), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=600)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=60).stdout
    rows = []
    for line in out.split("\n"):
        if line.strip():
            dt, mode, multi, bg, cap, b, bps = line.split()
            rows.append(dict(dt=dt, mode=int(mode), multi=bool(int(multi)), bg=bool(int(bg)), cap=int(cap),
                             bytes=int(b), blocks=int(bps)))
    return rows


def test_every_instantiation_fits_its_blocks_per_sm(layout_rows):
    assert len(layout_rows) == 3 * 18
    for r in layout_rows:
        need = r["blocks"] * (r["bytes"] + BLOCK_RESERVED)
        assert need <= SM_SHARED, f"{r}: {r['blocks']} blocks need {need} B of shared memory"


def test_forward_kernels_leave_l1_its_60_kb(layout_rows):
    fwd = [r for r in layout_rows if r["mode"] in (0, 3)]   # kFwd, kFusedFwd
    assert len(fwd) == 3 * 6
    for r in fwd:
        assert r["blocks"] == (5 if r["multi"] or r["bg"] else 6), r
        need = r["blocks"] * (r["bytes"] + BLOCK_RESERVED)
        assert need <= FORWARD_CARVEOUT, f"{r}: {need} B leave less than 60 KB of L1"


def test_reverse_kernel_runs_eight_blocks(layout_rows):
    rev = [r for r in layout_rows if r["mode"] == 4 and not r["multi"]]
    assert rev and all(r["blocks"] == 8 for r in rev)
