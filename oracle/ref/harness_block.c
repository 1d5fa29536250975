/* Read access to the reference's block storage (lsd_mkb/lad_block), the
 * storage the MKB solver uses for DG problems (DOF blocks of one element each,
 * lar_allocate_SM_and_LV_block, las_block_intf.c).  Each block row b keeps its
 * diagonal block Dia (Ndof x Ndof) and one off-diagonal block Aux[k] per
 * neighbour Lngb[1 + k] (Ndof_b x Ndof_neighbour); both column-major, leading
 * dimension the row block's Ndof (las_block_intf.c:362-520).
 *
 * refh_block_crs expands them to a scalar CRS over global dofs (Posg + local)
 * with every entry of every block present and columns sorted; with NULL
 * outputs it returns the entry count only.  Separate from harness.c because
 * the block and CRS headers cannot be included together. */
#include <stdio.h>
#include <stdlib.h>
#include "lah_intf.h"
#include "lah_block.h"

static int cmp_posg(const void *a, const void *b)
{
  const int *x = (const int *)a, *y = (const int *)b;
  return (x[0] > y[0]) - (x[0] < y[0]);
}

int refh_block_crs(int id, int *nrdof, int *row_ptr, int *col_ind, double *val, double *rhs)
{
  itt_matrices *m;
  int b, nnz = 0, row = 0;
  if (id < 0 || id >= itv_nr_matrices) return -1;
  m = &itv_matrices[id];
  if (nrdof) *nrdof = m->Nrdofgl;
  if (row_ptr) row_ptr[0] = 0;
  for (b = 1; b <= m->Nrblocks; b++) {
    itt_blocks *B = m->Block[b];
    int nn, k, r, c, q;
    int cols[2 * 64];
    if (B->Lngb == NULL) continue;
    nn = B->Lngb[0];
    if (nn + 1 > 64) return -2;
    /* (posg, neighbour index; -1 = diagonal) sorted by posg */
    cols[0] = B->Posg; cols[1] = -1;
    for (k = 0; k < nn; k++) { cols[2 * (k + 1)] = m->Block[B->Lngb[1 + k]]->Posg; cols[2 * (k + 1) + 1] = k; }
    qsort(cols, nn + 1, 2 * sizeof(int), cmp_posg);
    for (r = 0; r < B->Ndof; r++) {
      for (q = 0; q <= nn; q++) {
        int k2 = cols[2 * q + 1];
        itt_blocks *C = k2 < 0 ? B : m->Block[B->Lngb[1 + k2]];
        const double *blk = k2 < 0 ? B->Dia : B->Aux[k2];
        for (c = 0; c < C->Ndof; c++) {
          if (col_ind) col_ind[nnz] = C->Posg + c;
          if (val) val[nnz] = blk[c * B->Ndof + r];
          nnz++;
        }
      }
      if (row_ptr) row_ptr[row + 1] = nnz;
      if (rhs) rhs[B->Posg + r] = B->Rhs[r];
      row++;
    }
  }
  return nnz;
}
