"""Shared-memory budget of every render_kernel instantiation, checked on the host.

The kernels' speed depends on how many blocks share an SM and on how much of the SM's 256 KB of
shared memory plus L1 is left to L1.  A host-only program compiled against render_core.cuh prints,
for each instantiation, the dynamic shared memory per block (warp_smem_floats of its SmemLayout,
times the block's warps) and the blocks per SM its __launch_bounds__ asks for, and carves a warp's
slice on a host buffer with the kernel's own carve().  The test holds:
  * every instantiation: its blocks fit the 228 KB an SM offers (each block also reserves 1 KB);
  * the forward kernels (six blocks; five for the MSI background's and the batch launch's): their
    blocks fit the 196 KB carve-out, which leaves 60 KB of L1 for the row copies and gathers;
  * every carved region lies inside the slice, no two overlap, and the regions moved as int4 /
    float4 words (the tile, the corner links, the optical depths, the colour cache) start on
    16-byte boundaries.
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
#include <vector>
using namespace svx::rk;

struct Region { const char* name; const void* p; size_t bytes; size_t align; };

// carve() on a host buffer: regions inside the slice, pairwise disjoint, aligned
template <typename ShT, int MODE, bool five>
void check_carve(const char* dt, int scap) {
  const SmemLayout L = smem_layout<ShT, MODE, five>(27, scap);
  const int nf = warp_smem_floats(L);
  std::vector<float4> buf(nf / 4 + 1);
  float* base = reinterpret_cast<float*>(buf.data());
  const WarpSmem s = carve(base, L);
  const size_t nrow = L.rows > 0 ? kMaxRows : 0;
  std::vector<Region> r = {
      {"tile", s.tile, 4u * tile_floats(L.rs, L.rows, L.fc), 16},
      {"links", s.links, 4u * 256, 16},
      {"slot", s.slot, 4u * kSlots * L.ss, 4},
      {"rowlink", s.rowlink, 4u * nrow, 4},
      {"rowdst", s.rowdst, 2u * nrow, 2},
      {"run_lane", s.run_lane, 4u * kSlots, 4},
      {"run_l", s.run_l, 12u * kSlots, 4},
      {"basis", s.basis, 4u * 12, 4}};
  if (L.pc) r.push_back({"pc", s.pc, 4u * 32, 16});
  if (L.walk) r.push_back({"run_walk", s.run_walk, 4u * kSlots, 4});
  if (L.plan) {
    r.push_back({"run_need", s.run_need, (size_t)kSlots, 1});
    r.push_back({"run_delta", s.run_delta, (size_t)kSlots, 1});
  }
  if (L.ckpt) {
    r.push_back({"ck_t", s.ck_t, 4u * kNumCkpt, 4});
    r.push_back({"ck_lt", s.ck_lt, 4u * kNumCkpt, 4});
    r.push_back({"ck_idx", s.ck_idx, 4u * kNumCkpt, 4});
    r.push_back({"tmp_t", s.tmp_t, 4u * kMaxStride, 4});
    r.push_back({"tmp_lt", s.tmp_lt, 4u * kMaxStride, 4});
    r.push_back({"tmp_idx", s.tmp_idx, 4u * kMaxStride, 4});
  }
  if (scap > 0) r.push_back({"col", s.col, 16u * scap, 16});
  const uintptr_t lo = reinterpret_cast<uintptr_t>(base), hi = lo + 4u * (size_t)nf;
  const char* bad = nullptr;
  char why[160];
  for (size_t i = 0; i < r.size() && !bad; ++i) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(r[i].p);
    if (r[i].bytes == 0) continue;
    if (a < lo || a + r[i].bytes > hi) { bad = r[i].name; snprintf(why, sizeof why, "outside the slice"); }
    else if (a % r[i].align) { bad = r[i].name; snprintf(why, sizeof why, "not %zu-byte aligned", r[i].align); }
    for (size_t j = 0; j < i && !bad; ++j) {
      const uintptr_t b = reinterpret_cast<uintptr_t>(r[j].p);
      if (r[j].bytes && a < b + r[j].bytes && b < a + r[i].bytes) {
        bad = r[i].name;
        snprintf(why, sizeof why, "overlaps %s", r[j].name);
      }
    }
  }
  if (bad) printf("carve %s %d %d %d FAIL %s %s\n", dt, MODE, (int)five, scap, bad, why);
  else printf("carve %s %d %d %d ok\n", dt, MODE, (int)five, scap);
}

template <typename ShT, int MODE, bool MULTI, bool BG>
void row(const char* dt, int cap) {
  constexpr bool five = MULTI || BG;
  const int scap = (MODE == kFusedFwd || MODE == kFusedRev) ? 0 : cap;
  const size_t b = sizeof(float) * (size_t)warp_smem_floats(smem_layout<ShT, MODE, five>(27, scap)) * kWarps;
  printf("%s %d %d %d %d %zu %d\n", dt, MODE, (int)MULTI, (int)BG, scap, b, blocks_per_sm_bound(MODE, MULTI, BG));
  check_carve<ShT, MODE, five>(dt, scap);
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
        if line.startswith("carve "):
            rows.append(dict(carve=line))
        elif line.strip():
            dt, mode, multi, bg, cap, b, bps = line.split()
            rows.append(dict(dt=dt, mode=int(mode), multi=bool(int(multi)), bg=bool(int(bg)), cap=int(cap),
                             bytes=int(b), blocks=int(bps)))
    return rows


def test_every_instantiation_fits_its_blocks_per_sm(layout_rows):
    layout_rows = [r for r in layout_rows if "carve" not in r]
    assert len(layout_rows) == 3 * 18
    for r in layout_rows:
        need = r["blocks"] * (r["bytes"] + BLOCK_RESERVED)
        assert need <= SM_SHARED, f"{r}: {r['blocks']} blocks need {need} B of shared memory"


def test_forward_kernels_leave_l1_its_60_kb(layout_rows):
    fwd = [r for r in layout_rows if "carve" not in r and r["mode"] in (0, 3)]   # kFwd, kFusedFwd
    assert len(fwd) == 3 * 6
    for r in fwd:
        assert r["blocks"] == (5 if r["multi"] or r["bg"] else 6), r
        need = r["blocks"] * (r["bytes"] + BLOCK_RESERVED)
        assert need <= FORWARD_CARVEOUT, f"{r}: {need} B leave less than 60 KB of L1"


def test_reverse_kernel_runs_eight_blocks(layout_rows):
    rev = [r for r in layout_rows if "carve" not in r and r["mode"] == 4 and not r["multi"]]
    assert rev and all(r["blocks"] == 8 for r in rev)


def test_carved_regions_are_inside_disjoint_and_aligned(layout_rows):
    carves = [r["carve"] for r in layout_rows if "carve" in r]
    assert len(carves) == 3 * 18
    bad = [c for c in carves if not c.endswith(" ok")]
    assert not bad, bad
