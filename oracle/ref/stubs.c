/*
 * stubs.c - test infrastructure only.  Entry points the linked reference
 * modules reference but the integrate/assemble/GMRES path never reaches
 * (result files, images, direct solvers, multigrid levels, projections).
 * Kept in a translation unit without the reference headers so the stubs
 * need not repeat the full prototypes.
 */
#include <stdio.h>
#include <stdlib.h>

/* I/O and image stubs (not on the integrate/assemble/solve path) */
int utr_io_result_ctrl_pts_nr(void) { return 0; }
int utr_io_result_ctrl_pt_get_coords(int a, double *b) { (void)a; (void)b; return 0; }
int utr_io_write_img_to_pbm() { return 0; }
int utr_io_result_ctrl_pts_set_sol_len(int a) { (void)a; return 0; }
int utr_io_result_ctrl_pts_set_filename() { return 0; }
int utr_io_result_ctrl_pts_read_file() { return 0; }
int utr_io_result_ctrl_pt_set_elemID() { return 0; }
int utr_io_result_ctrl_pt_get_elemID() { return 0; }
int utr_io_result_add_ctrl_pt_values() { return 0; }
int utr_io_result_add_column() { return 0; }
int utr_io_initialize_mesh() { return 0; }
int utr_io_decompress_file() { return 0; }
int utr_io_compress_file() { return 0; }

/* direct solvers are not linked (only GMRES is on the path) */
int lsr_mkb_direct_init() { fprintf(stderr, "direct solver not linked\n"); exit(-1); }
int lsr_mkb_direct_create() { fprintf(stderr, "direct solver not linked\n"); exit(-1); }
int lsr_mkb_direct_solve() { fprintf(stderr, "direct solver not linked\n"); exit(-1); }
int lsr_mkb_direct_free() { return 0; }
int lsr_mkb_direct_destroy() { return 0; }

double *pdr_select_el_coeff() { fprintf(stderr, "obsolete pdr_select_el_coeff\n"); exit(-1); }
int pdr_comp_stiff_mat_uncon() { fprintf(stderr, "pdr_comp_stiff_mat_uncon not linked\n"); exit(-1); }
int pdr_get_list_ent_coarse() { fprintf(stderr, "multigrid levels not linked\n"); exit(-1); }
int pdr_dof_ent_sons() { fprintf(stderr, "multigrid levels not linked\n"); exit(-1); }
int pdr_L2_proj_sol() { fprintf(stderr, "projection not linked\n"); exit(-1); }
int pdr_create_exchange_tables() { return 1; }

/* serial builds: a few reference files call the OpenMP runtime without an
   _OPENMP guard; weak definitions give the one-thread answers and yield to
   libgomp in the OpenMP build */
__attribute__((weak)) int omp_get_num_threads(void) { return 1; }
__attribute__((weak)) int omp_get_thread_num(void) { return 0; }
__attribute__((weak)) int omp_get_max_threads(void) { return 1; }
__attribute__((weak)) void omp_set_nested(int n) { (void)n; }
