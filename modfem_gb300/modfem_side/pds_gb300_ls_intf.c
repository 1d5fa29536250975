/*
 * pds_gb300_ls_intf.c - the ModFEM side of libmodfem_gb300 for the
 * convection-diffusion problem module with standard linear prisms.
 *
 * It provides pdr_create_assemble_stiff_mat (include/pdh_intf.h:230-249),
 * the call sir_solve makes once per level after lsr_mkb_clear_matrix
 * (sid_mkb/sis_mkb_intf.c:2058), and forwards it to
 * gbfem_create_assemble_stiff_mat on the GPU instead of the CPU driver
 * utr_create_assemble_stiff_mat (utd_util/uts_ls_intf.c:3368-4322).  Compile
 * it into the problem module in place of the body in
 * pdd_conv_diff/linear_solver_interface/pds_conv_diff_ls_intf.c:253 and link
 * libmodfem_gb300.so; sir_create's lists, colours and tables, MKB's CRS
 * matrix (lad_crs, itv_crs_matrices) and the solver stay as they are.
 *
 * On the first call it gathers, through the module interfaces the CPU
 * element loop uses:
 *   - node coordinates (mmr_node_coor) and element vertices in
 *     mmr_el_node_coor order for every element and node id 1..max id
 *     (refined parents included: only active elements are in the entity
 *     lists; meshes refined without derefinement leave no free ids);
 *   - the constrained (hanging) vertices of a refined mesh, the vertices
 *     without a dof (apr_get_ent_pdeg == 0), with their constraining
 *     vertices from apr_get_constr_data;
 *   - the boundary faces with a Dirichlet flag (pdr_get_bc_type), their first
 *     neighbour and its side (mmr_fa_eq_neig);
 *   - the CRS structure of MKB's matrix;
 * and on every call the coefficients per element, from pdr_el_coeff at the
 * element's first vertex (the GPU path takes coefficients constant per
 * element: the 9 diffusion entries and the source), the Dirichlet value
 * from pdr_fa_coeff on the first Dirichlet face and the penalty of the
 * conv-diff weak form (1e7, pds_conv_diff_weakform_std.c:480).
 * The entity lists and tables stay cached on the device between calls
 * (GBFEM_OPT_CACHE_TABLES): gbfem_shim_reset (call it from sir_free) voids
 * them and the context.
 *
 * Returns 1 like the reference's function, < 0 with the library's message on
 * stderr when the GPU path fails.
 */
#include <stdio.h>
#include <stdlib.h>

#include "aph_intf.h"
#include "lah_crs.h"
#include "mmh_intf.h"
#include "pdh_control_intf.h"
#include "pdh_conv_diff.h"
#include "pdh_intf.h"

#include "modfem_gb300.h"

static gbfem_ctx gbs_ctx = NULL;
static int gbs_nel = 0, gbs_nno = 0;
static double *gbs_D = NULL;

/* the matrix MKB assembles into: one problem, the first CRS matrix */
static itt_crs_matrices *gbs_matrix(void) { return &itv_crs_matrices[0]; }

static int gbs_fail(const char *where)
{
  fprintf(stderr, "gbfem shim: %s: %s\n", where, gbfem_last_error());
  return -1;
}

/* Mesh, boundary faces and CRS structure, once per mesh. */
static int gbs_setup(int Problem_id)
{
  const int mesh_id = pdr_ctrl_i_params(Problem_id, 2);
  const int nno = mmr_get_max_node_id(mesh_id), nel = mmr_get_max_elem_id(mesh_id);
  int fa = 0, nbf = 0, i, j;
  double *xyz = malloc(3 * sizeof(double) * (size_t)nno);
  int *el = malloc(6 * sizeof(int) * (size_t)nel);
  int *fid, *fel, *fside, *fbc;
  if (!xyz || !el) return -1;
  for (i = 1; i <= nno; i++) mmr_node_coor(mesh_id, i, &xyz[3 * (i - 1)]);
  for (i = 1; i <= nel; i++) {
    int nodes[MMC_MAXELVNO + 1];
    mmr_el_node_coor(mesh_id, i, nodes, NULL);
    for (j = 0; j < 6; j++) el[6 * (i - 1) + j] = nodes[j + 1] - 1;
  }
  while ((fa = mmr_get_next_face_all(mesh_id, fa)) != 0) {
    if (mmr_fa_status(mesh_id, fa) == MMC_ACTIVE && pdr_get_bc_type(mmr_fa_bc(mesh_id, fa)) == PDC_BC_DIRI) nbf++;
  }
  fid = malloc(sizeof(int) * (size_t)(nbf + 1));
  fel = malloc(sizeof(int) * (size_t)(nbf + 1));
  fside = malloc(sizeof(int) * (size_t)(nbf + 1));
  fbc = malloc(sizeof(int) * (size_t)(nbf + 1));
  nbf = 0;
  fa = 0;
  while ((fa = mmr_get_next_face_all(mesh_id, fa)) != 0) {
    int bc, neig[2], sides[2];
    if (mmr_fa_status(mesh_id, fa) != MMC_ACTIVE) continue;
    bc = mmr_fa_bc(mesh_id, fa);
    if (pdr_get_bc_type(bc) != PDC_BC_DIRI) continue;
    mmr_fa_eq_neig(mesh_id, fa, neig, sides, NULL);
    fid[nbf] = fa;
    fel[nbf] = abs(neig[0]) - 1;
    fside[nbf] = sides[0];
    fbc[nbf] = bc;
    nbf++;
  }
  if (gbfem_create(&gbs_ctx, 0) < 0) return gbs_fail("gbfem_create");
  if (gbfem_set_mesh(gbs_ctx, nno, xyz, nel, GBFEM_PRISM, el, nbf, fid, fel, fside, fbc) < 0)
    return gbs_fail("gbfem_set_mesh");
  {
    const int field_id = pdr_ctrl_i_params(Problem_id, 3);
    int *cv = malloc(sizeof(int) * (size_t)nno), *cn = malloc(sizeof(int) * (size_t)nno);
    int *cp = malloc(4 * sizeof(int) * (size_t)nno), nc = 0, rc;
    if (!cv || !cn || !cp) return -1;
    for (i = 1; i <= nno; i++) {
      int constr[5];
      if (mmr_node_status(mesh_id, i) != MMC_ACTIVE || apr_get_ent_pdeg(field_id, APC_VERTEX, i) != 0) continue;
      apr_get_constr_data(field_id, i, APC_VERTEX, constr, NULL);
      cv[nc] = i - 1;
      cn[nc] = constr[0];
      for (j = 0; j < 4; j++) cp[4 * nc + j] = j < constr[0] ? constr[j + 1] - 1 : -1;
      nc++;
    }
    rc = gbfem_set_constraints(gbs_ctx, nc, cv, cn, cp);
    free(cv);
    free(cn);
    free(cp);
    if (rc < 0) return gbs_fail("gbfem_set_constraints");
  }
  {
    itt_crs_matrices *m = gbs_matrix();
    if (gbfem_set_crs_structure(gbs_ctx, m->Nrdofgl, NULL, m->Nnz, m->crs_row_ptr, m->crs_col_ind) < 0)
      return gbs_fail("gbfem_set_crs_structure");
  }
  gbfem_set_option(gbs_ctx, GBFEM_OPT_CACHE_TABLES, 1);
  free(xyz);
  free(el);
  free(fid);
  free(fel);
  free(fside);
  free(fbc);
  gbs_nel = nel;
  gbs_nno = nno;
  gbs_D = malloc(9 * sizeof(double) * (size_t)nel);
  return gbs_D ? 0 : -1;
}

/* Coefficients per element (pdr_el_coeff at the element's first vertex) and
   the Dirichlet value; returns the source f. */
static double gbs_coefficients(int Problem_id, double *g_out)
{
  const int mesh_id = pdr_ctrl_i_params(Problem_id, 2);
  double f = 0.0, xloc[3] = {0.0, 0.0, -1.0};
  int e, fa = 0;
  for (e = 1; e <= gbs_nel; e++) {
    int nodes[MMC_MAXELVNO + 1];
    double coor[3 * MMC_MAXELVNO], m, b[3], t[3], c, l, q[3], s, *A = gbs_D + 9 * (size_t)(e - 1);
    mmr_el_node_coor(mesh_id, e, nodes, coor);
    pdr_el_coeff(Problem_id, e, mmr_el_groupID(mesh_id, e), 0.0, 1, xloc, NULL, NULL, NULL, NULL, coor, NULL,
                 NULL, NULL, NULL, NULL, NULL, NULL, NULL, &m, &A[0], &A[1], &A[2], &A[3], &A[4], &A[5], &A[6],
                 &A[7], &A[8], &b[0], &b[1], &b[2], &t[0], &t[1], &t[2], &c, &l, &q[0], &q[1], &q[2], &s);
    if (e == 1) f = s;
  }
  *g_out = 0.0;
  while ((fa = mmr_get_next_face_all(mesh_id, fa)) != 0) {
    const int bc = mmr_fa_bc(mesh_id, fa);
    if (mmr_fa_status(mesh_id, fa) == MMC_ACTIVE && pdr_get_bc_type(bc) == PDC_BC_DIRI) {
      int neig[2];
      double xc[3] = {0.0, 0.0, 0.0}, vn[3] = {0.0, 0.0, 1.0}, u[1] = {0.0}, ux[1] = {0.0}, uy[1] = {0.0};
      double uz[1] = {0.0}, anx, any, anz, bn, fval[1] = {0.0}, gval[1] = {0.0}, qn, vel;
      mmr_fa_eq_neig(mesh_id, fa, neig, NULL, NULL);
      pdr_fa_coeff(fa, bc, abs(neig[0]), 0, 0.0, 0.0, 1, xc, vn, u, ux, uy, uz, &anx, &any, &anz, &bn, fval,
                   gval, &qn, &vel);
      *g_out = fval[0];
      break;
    }
  }
  return f;
}

/* Voids the device context and cached tables (call from sir_free). */
void gbfem_shim_reset(void)
{
  if (gbs_ctx) gbfem_destroy(gbs_ctx);
  gbs_ctx = NULL;
  free(gbs_D);
  gbs_D = NULL;
  gbs_nel = gbs_nno = 0;
}

int pdr_create_assemble_stiff_mat(int Problem_id, int Level_id, int Comp_type, int *Pdeg_coarse_p,
                                  int Nr_int_ent, int *L_int_ent_type, int *L_int_ent_id, int Nr_colors_elems,
                                  int *L_color_index_elems, int Nr_colors_faces, int *L_color_index_faces,
                                  int *Asse_pos_first_dof_int_ent, int *Assembly_table, int Max_dofs_int_ent)
{
  itt_crs_matrices *m = gbs_matrix();
  double g = 0.0, f;
  if (!gbs_ctx && gbs_setup(Problem_id) < 0) return -1;
  f = gbs_coefficients(Problem_id, &g);
  {
    /* isotropic tensors (k I) go as k: the double-word element kernel
       takes them; full tensors take the FP64 tensor kernel */
    int e, iso = 1;
    for (e = 0; e < gbs_nel && iso; e++) {
      const double *A = gbs_D + 9 * (size_t)e;
      iso = A[1] == 0.0 && A[2] == 0.0 && A[3] == 0.0 && A[5] == 0.0 && A[6] == 0.0 && A[7] == 0.0 &&
            A[0] == A[4] && A[0] == A[8];
    }
    if (iso) {
      double *k = malloc(sizeof(double) * (size_t)(gbs_nel > 0 ? gbs_nel : 1));
      int rc;
      if (!k) return -1;
      for (e = 0; e < gbs_nel; e++) k[e] = gbs_D[9 * (size_t)e];
      rc = gbfem_set_coefficients(gbs_ctx, k, NULL, f, g, 1.0e7);
      free(k);
      if (rc < 0) return gbs_fail("gbfem_set_coefficients");
    } else if (gbfem_set_coefficients(gbs_ctx, NULL, gbs_D, f, g, 1.0e7) < 0) {
      return gbs_fail("gbfem_set_coefficients");
    }
  }
  if (gbfem_create_assemble_stiff_mat(gbs_ctx, Level_id, Comp_type, Pdeg_coarse_p, Nr_int_ent, L_int_ent_type,
                                      L_int_ent_id, Nr_colors_elems, L_color_index_elems, Nr_colors_faces,
                                      L_color_index_faces, Asse_pos_first_dof_int_ent, Assembly_table,
                                      Max_dofs_int_ent, m->crs_val, m->rhs) < 0)
    return gbs_fail("gbfem_create_assemble_stiff_mat");
  return 1;
}
