// Host driver for tests/test_block_ell.py: lays out a CSR matrix with the
// PCG's node-block sliced ELL (xg::block_ell_layout, no GPU), then forms
// y = A x from the layout alone -- the slots the CSR values map to, the
// block columns, the padded node-major x -- as the device SpMV reads them,
// and the rows the layout leaves to CSR chunks from those chunks.
#include <cstring>
#include <vector>

#include "../../xara_gb300/csrc/xg_internal.h"

extern "C" int ell_apply(int n, const int *rowptr, const int *colidx, const double *vals, int nblk,
                         const int *blk_start, int cap, const double *x, double *y,
                         int *kb_out, int *chunked_rows, int *slot_clash) {
  xg::BlockEll h;
  const int kb = xg::block_ell_layout(n, rowptr, colidx, nblk, blk_start, cap, h);
  *kb_out = kb;
  *chunked_rows = 0;
  *slot_clash = 0;
  if (!kb) return 0;
  const int ks = kb == 3 ? 4 : kb;
  std::vector<double> packed((size_t)h.off.back() * kb * kb, 0.0);
  std::vector<char> used(packed.size(), 0);
  for (int q = 0; q < rowptr[n]; q++) {
    if (h.pos[q] < 0) continue;
    if (used[h.pos[q]]++) *slot_clash += 1;
    packed[h.pos[q]] = vals[q];
  }
  std::vector<double> xp((size_t)nblk * ks, 0.0);
  for (int j = 0; j < nblk; j++)
    for (int b = 0; b < blk_start[j + 1] - blk_start[j]; b++) xp[(size_t)j * ks + b] = x[blk_start[j] + b];
  std::memset(y, 0, sizeof(double) * n);
  for (int i = 0; i < nblk; i++) {
    const int m = blk_start[i + 1] - blk_start[i];
    if (h.len[i] > cap) continue;
    const long base = h.off[i / 32];
    const int lane = i % 32;
    for (int a = 0; a < m; a++) {
      double s = 0.0;
      for (int k = 0; k < h.len[i]; k++) {
        const int j = h.cols[base + 32L * k + lane];
        for (int b = 0; b < kb; b++)
          s += packed[base * kb * kb + ((long)(k * kb + a) * kb + b) * 32 + lane] *
               xp[(size_t)j * ks + b];
      }
      y[blk_start[i] + a] = s;
    }
  }
  // the long node rows, from their chunks of CSR entries
  for (size_t r = 0; r + 1 < h.long_chunk0.size(); r++) {
    *chunked_rows += 1;
    for (int c = h.long_chunk0[r]; c < h.long_chunk0[r + 1]; c++) {
      const int row = h.chunk_row[c];
      const int e = std::min(h.chunk_beg[c] + 512, rowptr[row + 1]);
      for (int q = h.chunk_beg[c]; q < e; q++) y[row] += vals[q] * x[colidx[q]];
    }
  }
  return 0;
}
