/* lakcluster_gb300.h -- C ABI of the GB300 (sm_103a) implementation of
 * lakcluster's binary case/control loop-counting pass (bcc).
 *
 * The data model is the reference's, byte for byte, so a caller built against
 * the reference headers can link this library in place of the CPU kernels:
 *   struct M_handle  -- dir_h/M_handle.h:1-27   (packed +/-1 bit matrix + masks)
 *   struct L_handle  -- dir_h/L_handle.h:1-11   (FP64 output, lf[r + c*row_stride])
 *
 * Every wrap_* entry point keeps the reference's signature and semantics:
 * *output_p == NULL  -> the callee allocates the L_handle (malloc here, the
 * reference uses its bump arena); otherwise the callee checks its length and
 * zero-fills it; the return value is the output length.  The thread arguments
 * (tidx, vpra, thread_in) are accepted for source compatibility: the work is
 * enqueued on the library's CUDA stream and the call returns after the result
 * is back in host memory (the reference's later pthread join becomes a no-op).
 *
 * Errors: no reference entry point returns a status, so device and argument
 * errors are recorded in a library-global status read by lakgb_last_error();
 * fatal conditions abort the way the reference does (exit with RET_* codes).
 */
#ifndef LAKCLUSTER_GB300_H
#define LAKCLUSTER_GB300_H

#include <stdio.h>
#include <pthread.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LAKGB_FNAMESIZE (4096 + 256)

/* dir_h/M_handle.h:1-27 -- identical field order and types. */
struct M_handle {
  unsigned char *mark;
  int header_length;
  char A_name[LAKGB_FNAMESIZE];
  FILE *A_fp; unsigned char *Ara;
  int bitj;
  int nrows; int ncols;
  int nrows_extend; int ncols_extend;
  long long int rpop_b; long long int rpop_j;
  long long int cpop_b; long long int cpop_j;
  unsigned char *wX;
  unsigned char *mr_b; unsigned char *mr_j;
  unsigned char *mc_b; unsigned char *mc_j;
  double *rsum;
  unsigned int *m_a_;
  unsigned int *m_b_;
  unsigned int *n_a_;
  unsigned int *n_b_;
  unsigned long mr_length; unsigned long mc_length;
  unsigned long cc_length;
  unsigned long wt_length;
  unsigned char *wt;
  unsigned long long int length_total;
  int ncols_per_z;
  double max_d; double min_d; double mlt_d;
};

/* dir_h/L_handle.h:1-11 -- identical field order and types. */
struct L_handle {
  unsigned long long int length;
  double *lf;
  int spacing_row; unsigned long long int row_stride;
  int spacing_col; unsigned long long int col_stride;
  int spacing_lyr; unsigned long long int lyr_stride;
};

/* Constants with the reference's values (dir_h/lakcluster_header.h). */
#define LAKGB_TYPE_p0 0
#define LAKGB_TYPE_pm 1
#define LAKGB_TYPE_00 2
#define LAKGB_SPACING_b 0
#define LAKGB_SPACING_j 1
#define LAKGB_SPACING_a 2
#define LAKGB_AJDK_TOT 15
#define LAKGB_POPLENGTH 1920

/* ---------------------------------------------------------------------------
 * Kernel entry points (drop-in replacements).
 * ------------------------------------------------------------------------- */

/* Centred, D-weighted +/-1 Gram (An - e*alpha) diag(D) (Zt - alpha*e) over the
 * current columns mc_j of M_An; TYPE_00 gives the masked AND count instead.
 * Replaces wrap_AnZt_vv__run, dir_c/AnZt_vv.c:185 (kernel get_AnZt_vv__run,
 * AnZt_vv.c:5-183). */
int wrap_AnZt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                      int output_spacing_r, int output_spacing_c,
                      struct M_handle *M_An, struct M_handle *M_Zn, double *A_ajdk,
                      struct L_handle *lf_An_ajdk, struct L_handle *lf_Zn_ajdk,
                      struct L_handle **output_AnZt_p);

/* Symmetric variant with Zn == An.  Replaces wrap_AnAt_vv__run,
 * dir_c/AnAt_vv.c:157 (kernel AnAt_vv.c:5-155). */
int wrap_AnAt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                      int output_spacing_r, int output_spacing_c,
                      struct M_handle *M_An, struct M_handle *M_Zn, double *A_ajdk,
                      struct L_handle *lf_An_ajdk, struct L_handle *lf_Zn_ajdk,
                      struct L_handle **output_AnAt_p);

/* Masked row sums An*1 (TYPE_pm: +/-1, TYPE_00: 0/1).  Replaces
 * wrap_An_v__run, dir_c/An_v.c:59 (kernel An_v.c:5-57). */
int wrap_An_v__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                   int output_spacing_r, struct M_handle *M_An,
                   struct L_handle **output_An_v_p);

/* Row products An*diag(alpha^j D^k) for the 15 (j,k) pairs.  Replaces
 * wrap_An_ajdk_v, dir_c/An_ajdk_v.c:365 (kernel An_ajdk_v.c:272-363). */
int wrap_An_ajdk_v(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                   int output_spacing_r, struct M_handle *M_An, double *A_ajdk,
                   struct L_handle **output_An_ajdk_p);

/* Quantise an FP64 matrix YnWt (rows mr_*, columns mc_*) into 1+b_mlt bit
 * planes over the Yn rows: plane 0 marks the retained rows, planes
 * 1..b_mlt hold the bits of floor(mlt*(x-min)) cropped to [1, D_MLT-1]
 * (D_MLT = 2^b_mlt unless set with lakgb_set_d_mlt).  trm_flag = 1 reads
 * YnWt transposed.  *M_X_p must be pre-allocated (the reference allocates it
 * when NULL; this library requires it).  Replaces wrap_xcalc,
 * dir_c/xcalc.c:248 (kernel get_xcalc, xcalc.c:41-246). */
void wrap_xcalc(int *tidx, void **vpra, pthread_t *thread_in, unsigned char *mr_j,
                unsigned char *mr_b, unsigned char *mc_j, unsigned char *mc_b,
                struct L_handle *lf_YnWt, double *YnWt, int *Yn_nrows_p, int *Wn_nrows_p,
                struct M_handle **M_X_p, int *b_mlt_p, int trm_flag);

/* out[na, t] = sum_w sum_z (At_na - alpha) diag(T_t) (YnWt)_w diag(S_t) (Zt - alpha)
 * evaluated through the bit planes M_YnWt made by wrap_xcalc (the loop product
 * behind the column scores).  Replaces wrap_At_T_YnWt_S_Zn_ww__run,
 * dir_c/At_T_YnWt_S_Zn_ww.c:435 (kernel At_T_YnWt_S_Zn_ww.c:5-433). */
int wrap_At_T_YnWt_S_Zn_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a,
                                int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                                struct M_handle *M_Yn, struct M_handle *M_Wn,
                                struct M_handle *M_St, struct M_handle *M_Zt, double *A_ajdk,
                                struct M_handle *M_YnWt,
                                struct L_handle **output_At_T_YnWt_S_Zn_ww_p);

/* out[na, s] = sum_z AnZt[na,z] * S[s,z] * YnWt[na,z] (the loop product behind
 * the row scores).  Replaces wrap_AnZt_S_WnYt_vv__run,
 * dir_c/AnZt_S_WnYt_vv.c:103 (kernel AnZt_S_WnYt_vv.c:5-101). */
int wrap_AnZt_S_WnYt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                             int output_spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                             struct M_handle *M_Zn, struct L_handle *lf_AnZt,
                             struct L_handle *lf_YnWt, struct L_handle **output_p);

/* out[na, s] = An_na . ZtSn[:, s] evaluated through the bit planes M_ZtSn made
 * by wrap_xcalc.  Replaces wrap_An_ZtSn_ww__run, dir_c/An_ZtSn_ww.c:110
 * (kernel An_ZtSn_ww.c:5-108). */
int wrap_An_ZtSn_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a,
                         int spacing_s, struct M_handle *M_An, struct L_handle *lf_ZtSn,
                         struct M_handle *M_ZtSn, struct M_handle *M_St,
                         struct L_handle **output_An_ZtSn_ww_p);

/* out[na, ny, t] = (At_na - alpha) diag(T_t) (Yt_ny - alpha)^T over the rows
 * (a SNP x SNP x covariate product).  Replaces wrap_AtTYn_vv__run,
 * dir_c/AtTYn_vv.c:204 (kernel AtTYn_vv.c:5-202). */
int wrap_AtTYn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                       int output_spacing_y, int output_spacing_t, struct M_handle *M_At,
                       struct M_handle *M_Tt, struct M_handle *M_Yt, double *A_ajdk,
                       double *Y_ajdk, struct L_handle *lf_AtTn, struct L_handle *lf_YtTn,
                       struct L_handle **output_AtTYn_p);

/* out[na, s] = sum_{ny,nw} AtTYn[na,ny,s] * D[ny] * ZtSWn[nw..,s] (contraction of
 * two AtTYn products).  Replaces wrap_AtTYn____WtSZn_vv__run,
 * dir_c/AtTYn____WtSZn_vv.c:117 (kernel AtTYn____WtSZn_vv.c:5-115). */
int wrap_AtTYn____WtSZn_vv__run(int *tidx, void **vpra, pthread_t *thread_in,
                                int output_spacing_a, int output_spacing_s,
                                struct M_handle *M_At, struct M_handle *M_Tt,
                                struct M_handle *M_Yt, struct M_handle *M_Wt,
                                struct M_handle *M_St, struct M_handle *M_Zt, double *Y_ajdk,
                                struct L_handle *lf_AtTYn, struct L_handle *lf_ZtSWn,
                                struct L_handle **output_p);

/* The SNP x SNP x covariate product with Yt = At, each pair computed once and
 * stored at both (na, ny) and (ny, na).  Replaces wrap_AtTAn_vv__run,
 * dir_h/lakcluster_header.h:376 (kernel dir_c/AtTAn_vv.c:5-172). */
int wrap_AtTAn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                       int output_spacing_y, int output_spacing_t, struct M_handle *M_At,
                       struct M_handle *M_Tt, struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk,
                       struct L_handle *lf_AtTn, struct L_handle *lf_YtTn, struct L_handle **output_AtTAn_p);

/* The loop product element by element from the FP64 YnWt (no quantisation):
 * the reference's ground truth for wrap_At_T_YnWt_S_Zn_ww__run.  Replaces
 * wrap_At_T_YnWt_S_Zn_vv__run, dir_c/At_T_YnWt_S_Zn_vv.c:87 (kernel :5-85). */
int wrap_At_T_YnWt_S_Zn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                int output_spacing_s, struct M_handle *M_At, struct M_handle *M_Tt,
                                struct M_handle *M_St, struct M_handle *M_Zt, double *A_ajdk,
                                struct L_handle *lf_YnWt, struct L_handle **output_p);

/* (An - a) D ZtSWn D (Yt - a) element by element, An row paired with Yn row.
 * Replaces wrap_An_ZtSWn_Yt_vv__run, dir_c/An_ZtSWn_Yt_vv.c:131 (kernel :5-130). */
int wrap_An_ZtSWn_Yt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                             int output_spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                             struct M_handle *M_Yn, double *A_ajdk, double *Y_ajdk,
                             struct L_handle *lf_ZtSWn, struct L_handle **output_p);

/* The same product through bit planes: M_ZtSWn_[s] (one per retained St row)
 * holds the wrap_xcalc planes of that ZtSWn slice, ncols_per_z rows per
 * retained Wt row; the Wt handle supplies those rows' indices, An row paired
 * with Yn row.  Replaces wrap_An_ZtSWn_Yt_ww__run, dir_c/An_ZtSWn_Yt_ww.c:113
 * (kernel :5-111). */
int wrap_An_ZtSWn_Yt_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a, int spacing_s,
                             struct M_handle *M_An, struct M_handle *M_St, struct M_handle **M_ZtSWn_,
                             struct M_handle *M_Wt, struct M_handle *M_Yn, double *A_ajdk, double *Y_ajdk,
                             struct L_handle **output_An_ZtSWn_Yt_ww_p);

/* Dense FP64 copy of the retained entries of a bit matrix whose rows are SNPs
 * (At): (b - a_k) * sqrt(d_k), b = +1/-1 (TYPE_pm) or 1/0 (TYPE_00) and a_k,
 * d_k the A_ajdk terms of row k's SNP, or b alone when A_ajdk is NULL; rows
 * at output_spacing_r, columns at output_spacing_c; the whole output handle
 * is zeroed first.  Replaces wrap_M_At_to_L2_run, dir_c/M_Ax_to_L2.c:282
 * (kernel :137-280); used by the condense row strategy. */
int wrap_M_At_to_L2_run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag, int output_spacing_r,
                        int output_spacing_c, struct M_handle *M_At, double *A_ajdk, struct L_handle **output_L_p);

/* The same with SNPs as columns (An; a_k, d_k of column k's SNP).  Replaces
 * wrap_M_An_to_L2_run, dir_c/M_Ax_to_L2.c:102 (kernel :5-100). */
int wrap_M_An_to_L2_run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag, int output_spacing_r,
                        int output_spacing_c, struct M_handle *M_An, double *A_ajdk, struct L_handle **output_L_p);

/* FP64 product of two dense L_handles, C(i,j) = sum_k At(k,i) * Zt(k,j) over
 * At's row_stride values of k, each element one sum from +0 in ascending k
 * with the product and the sum rounded once (the order of the GSL CBLAS dgemm
 * the reference links).  Output rows follow At's column spacing, columns Zt's.
 * Replaces wrap_AnZt_mm__run, dir_c/AnZt_mm.c:86 (kernel :6-84). */
int wrap_AnZt_mm__run(int *tidx, void **vpra, pthread_t *thread_in, struct L_handle *lf_At, struct L_handle *lf_Zt,
                      struct L_handle **output_AnZt_p);

/* ---------------------------------------------------------------------------
 * Input pipeline: PLINK .bed to .b16 (bed_to_b16, dir_c/bed_to_b16.c:711-1355).
 * ------------------------------------------------------------------------- */

/* The conversion's thresholds (GLOBAL_snp_mss_threshold, _snp_maf_threshold,
 * _snp_I_opt_threshold, _pat_mss_threshold); _init sets the reference's
 * defaults 0.01, 0.25, 0.01, 0.04 (dir_c/lakcluster_ver18.c:158-161). */
struct lakgb_bed_params {
  double snp_mss_threshold, snp_maf_threshold, snp_I_opt_threshold, pat_mss_threshold;
};
void lakgb_bed_params_init(struct lakgb_bed_params *p);

/* A conversion's result: the kept SNPs (.bim indices) and patients (.fam
 * indices), three alleles per kept SNP (allele 3k+0 / 3k+1 / 3k+2 = nor / xor
 * / and of kept SNP k) with their frequency, maf, missing fraction and
 * relative entropy, the sorted allele order (row r of A_n is allele
 * allele_orig_from_sort[r]) and A_n itself: n_allele rows of row_bytes =
 * rup(n_pat_retain, 16) / 8 bytes, patients MSB first (the .b16 payload).
 * Arrays are malloc'ed; free with lakgb_bed_result_free. */
struct lakgb_bed_result {
  int n_snp, n_fam;
  int n_snp_retain, n_pat_retain, n_allele;
  long long row_bytes;
  int *snp_from_retain, *pat_from_retain, *allele_orig_from_sort;
  double *allele_frequency, *allele_maf, *allele_mss, *allele_I_opt;
  unsigned char *A_n;
};
void lakgb_bed_result_free(struct lakgb_bed_result *r);

/* bed_records: the .bed body (after its three magic bytes), n_snp records of
 * ceil(n_fam / 4) bytes.  params may be null (defaults).  Returns 0 on
 * success. */
int lakgb_bed_to_b16_mem(const unsigned char *bed_records, int n_snp, int n_fam,
                         const struct lakgb_bed_params *params, struct lakgb_bed_result *out);

/* The file form, replacing bed_to_b16 (GLOBAL_TEST_TYPE= bed_to_b16 with
 * GLOBAL_fname_{bed,bim,fam}_0in and GLOBAL_fname_{b16,bim,fam}_out; the same
 * .in statements work through lakgb_bcc_run_in_file): reads the .bed / .bim /
 * .fam, writes the .b16, one .bim line per allele in sorted order and the
 * kept patients' .fam lines, as the reference writes them.  Returns 0 on
 * success; lakgb_bed_last_error describes a failure. */
int lakgb_bed_to_b16(const char *bed, const char *bim, const char *fam, const char *b16_out,
                     const char *bim_out, const char *fam_out, const struct lakgb_bed_params *params);
int lakgb_bed_last_error(char *msg, int msg_len);

/* Merge n_file converted studies into one, replacing b16_merge
 * (dir_c/bed_to_b16.c:1659-1985; GLOBAL_TEST_TYPE= b16_merge with
 * GLOBAL_n_file, the GLOBAL_fname_{b16,bim,fam}_0in_ lists and
 * GLOBAL_fname_{b16,bim,fam}_out, also through lakgb_bcc_run_in_file): the
 * patients found in every study (FID and IID of the .fam lines, in sorted
 * order; the .fam lines of the first study), every study's allele rows
 * interleaved by the allele frequency of their .bim lines (ties to the lower
 * study), each row holding the common patients' bits.  Returns 0 on success;
 * lakgb_bed_last_error describes a failure. */
int lakgb_b16_merge(int n_file, const char *const *b16_in, const char *const *bim_in, const char *const *fam_in,
                    const char *b16_out, const char *bim_out, const char *fam_out);

/* ---------------------------------------------------------------------------
 * Whole solves.
 * ------------------------------------------------------------------------- */

/* Run the bcc solve described by a reference .in file (YnWt row strategy,
 * YnWt and / or ZtSWn column strategy, covariate T/S files, no Y/W matrices)
 * and write out_trace.txt, out_xdrop_a.txt and out_xdrop_b.txt into its
 * GLOBAL_DIR_NAME, exactly as the reference program does.  Replaces the
 * reference's main -> read_input -> lakcluster_driver path
 * (dir_c/lakcluster_ver18.c:238-330, dir_c/updateglobals.c:188-198,
 * dir_c/lakcluster_driver.c:14-251), including the scrambles named by
 * GLOBAL_scramble_num / GLOBAL_scramble_out_xdrop_ / GLOBAL_scramble_rseed_
 * (wrap_bcc_scramble, dir_c/R_init.c:165-290).  With GLOBAL_TEST_TYPE=
 * lakcluster_scorebox it runs the scorebox instead (lakcluster_scorebox,
 * dir_c/lakcluster_scorebox.c:103-271) over GLOBAL_scorebox_out_xdrop and
 * writes its five scorebox_r*n*_c*n*_*.mda arrays (dir_c/S_init.c:79-89).
 * Returns 0 on success; lakgb_bcc_last_error() describes a failure. */
int lakgb_bcc_run_in_file(const char *in_path);

/* In-memory form of the same solve (no reference counterpart: the reference
 * only reads files).  Rows are packed MSB-first, bit 1 = minor allele (+1);
 * each row occupies row_bytes bytes, of which the first rup(ncols,16)/8 are
 * used.  Masks are rup(n,16)/8 bytes, NULL = all rows / columns. */
struct lakgb_bcc_bin {
  int A_nrows; const unsigned char *A_rows; const unsigned char *A_mr_b;
  int Z_nrows; const unsigned char *Z_rows; const unsigned char *Z_mr_b;
  /* covariates (GLOBAL_T_t_name_ / GLOBAL_S_t_name_): one row of T_ncols bits
   * per case row (T_rows) and per control row (S_rows), rup(T_ncols,16)/8
   * bytes each; both NULL = one covariate column of ones (T_ncols 1) */
  const unsigned char *T_rows; const unsigned char *S_rows;
};
struct lakgb_bcc_problem {
  int ncols; long long row_bytes; const unsigned char *mc_b;
  int nbins; const struct lakgb_bcc_bin *bins;
  int B_MLT;         /* bits per quantised score (GLOBAL_B_MLT), 1..62 */
  double gamma;      /* elimination fraction (GLOBAL_gamma) */
  int gamma_type;    /* GLOBAL_gamma_type (0 = log) */
  int test_sparse;   /* GLOBAL_TEST_sparse (1 = estimate allele frequencies) */
  int Ireq;          /* GLOBAL_Ireq: > 0 scores each row / column by its Ireq-th
                        highest per-bin score (bcc_sumscores_srt); <= 0 sums bins */
  int T_ncols;       /* covariate columns of the bins' T_rows / S_rows (GLOBAL_T_n_cols) */
  double kappa_squared;  /* GLOBAL_kappa_squared: > 0 turns on the MDS correction
                            of the covariate columns (bcc_sumscores_ifT) */
  const char *QC_strategy;  /* GLOBAL_QC_strategy: "YnWt" (NULL), "ZtSWn", or both;
                               "YnWt store one" is accepted (same results as "YnWt") */
  const char *QR_strategy;  /* GLOBAL_QR_strategy: "YnWt" (NULL) or "YnWt condense" */
};
/* trace: 6 values per iteration (iteration, rows left, columns left, mean row
 * score, mean column score, bins with rows); xdrop_a / xdrop_b: 2 ints per
 * eliminated row or column, (row, -1) or (-1, column), in elimination order,
 * with a-space and b-space indices -- the contents of the reference's
 * out_trace.txt / out_xdrop_a.txt / out_xdrop_b.txt. */
struct lakgb_bcc_result {
  int iterations; double *trace;
  int n_xdrop; int *xdrop_a; int *xdrop_b;
};
void lakgb_bcc_problem_init(struct lakgb_bcc_problem *p);  /* reference defaults */
int lakgb_bcc_solve(const struct lakgb_bcc_problem *p, struct lakgb_bcc_result *r);
void lakgb_bcc_result_free(struct lakgb_bcc_result *r);
int lakgb_bcc_last_error(char *msg, int msg_len);

/* Many solves at once (no reference counterpart).  A server owns `workers`
 * host threads, each driving whole solves on its own CUDA stream, and admits a
 * submitted problem as soon as a worker is idle and its estimated device
 * footprint (lakgb_bcc_footprint) fits hbm_budget_bytes beside the solves
 * already running (<= 0: no budget); a problem that does not fit yet does not
 * hold back smaller ones submitted after it.  submit copies the problem's
 * arrays; wait blocks for one result (ownership passes to the caller; free it
 * with lakgb_bcc_result_free) and reports {queueing, solving, total} seconds.
 * Each result equals the same problem solved alone. */
struct lakgb_server;
struct lakgb_server *lakgb_server_create(int workers, long long hbm_budget_bytes);
long long lakgb_server_submit(struct lakgb_server *s, const struct lakgb_bcc_problem *p);
/* As submit, with a deadline `deadline_s` seconds after submission (<= 0:
 * none): a request still queued at its deadline fails with
 * LAKGB_E_DEADLINE, and a running one stops with that code at its next
 * elimination iteration. */
long long lakgb_server_submit_deadline(struct lakgb_server *s, const struct lakgb_bcc_problem *p,
                                       double deadline_s);
/* Returns the solve's status: 0, a lakgb_bcc_solve error code,
 * LAKGB_E_CANCELLED, LAKGB_E_DEADLINE, or -1 for an id that is not (or no
 * longer) known.  A request that failed fails alone: the others run on. */
int lakgb_server_wait(struct lakgb_server *s, long long id, struct lakgb_bcc_result *r, double *times3);
/* As wait, and the failure's message into msg (empty on success). */
int lakgb_server_wait_msg(struct lakgb_server *s, long long id, struct lakgb_bcc_result *r, double *times3,
                          char *msg, int msg_len);
/* Cancel a request: a queued one completes at once with LAKGB_E_CANCELLED;
 * a running one stops with that code at its next elimination iteration.
 * Returns 0, or -1 for an id that is not known or already finished. */
int lakgb_server_cancel(struct lakgb_server *s, long long id);
int lakgb_server_peak_concurrency(struct lakgb_server *s);
/* Stops the server: queued requests complete with LAKGB_E_CANCELLED (their
 * waiters return), running ones are cancelled and joined, and the call
 * returns once every thread inside lakgb_server_wait has left it.  No call on
 * `s` may start after destroy has begun. */
void lakgb_server_destroy(struct lakgb_server *s);
#define LAKGB_E_CANCELLED 6
#define LAKGB_E_DEADLINE 7
long long lakgb_bcc_footprint(const struct lakgb_bcc_problem *p);
/* High-water mark (bytes) of the device memory held by the library's
 * stream-ordered allocations (the device's default memory pool) since the
 * last reset; reset != 0 restarts it from the current use.  Lets a caller
 * compare lakgb_bcc_footprint with what a solve really held. */
long long lakgb_pool_high_water(int reset);
/* Solve n problems on a server of `workers` threads; returns the number that
 * failed (per-problem status in rcs, may be NULL). */
int lakgb_bcc_solve_many(const struct lakgb_bcc_problem *ps, int n, struct lakgb_bcc_result *rs, int *rcs,
                         int workers, long long hbm_budget_bytes);

/* ---------------------------------------------------------------------------
 * Device-resident entry points (no reference counterpart: the reference has
 * no device memory).  All pointers are device pointers; `stream` is a
 * cudaStream_t (NULL = the library's stream).  The call enqueues and returns.
 * ------------------------------------------------------------------------- */

/* One Gram launch on device-resident packed rows: the same arithmetic as
 * wrap_AnZt_vv__run (symmetric = 0) or wrap_AnAt_vv__run (symmetric = 1),
 * with the host-side argument preparation already done by the caller.
 * out[out_r[i] + out_c[k]*out_stride] = a0d1 - 2*S_ik - ((lfA[i]+lfZ[k]) - a2d1)
 * for TYPE_pm (S_ik = sum over 1920-bit blocks b of D[b]*popcount((A_i^Z_k)&mask)),
 * S_ik alone for TYPE_00; lfA/lfZ may be NULL, D may be NULL (unweighted). */
struct lakgb_gram_args {
  const unsigned char *wA; const unsigned int *a_rowb; int nA; long long a_row_bytes;
  const unsigned char *wZ; const unsigned int *z_rowb; int nZ; long long z_row_bytes;
  const unsigned char *mask; int P;
  const double *D; int type_flag;
  double a0d1; double a2d1;
  const double *lfA; const double *lfZ;
  const unsigned int *out_r; const unsigned int *out_c;
  const unsigned int *out_r2; const unsigned int *out_c2;
  long long out_stride; double *out;
  int symmetric;
  void *stream;
};
int lakgb_gram_device(const struct lakgb_gram_args *args);

/* .b16 bit-matrix transpose, file to file: the reference's wrap_transpose
 * (dir_c/binary_read.c:174) with its signature.  Reads fname_0in (header
 * bitj, n_row, n_col; n_col records of n_row bits padded to bitj), writes
 * fname_out (header bitj, n_col, n_row; n_row records of n_col bits, padding
 * bits zero), transposing on the GPU.  n_bytes_per_read (the reference's
 * workspace chunk) is accepted and not needed.  Errors: a printed warning,
 * as the reference does, and lakgb_last_error. */
void wrap_transpose(char *fname_0in, char *fname_out, int n_bytes_per_read);
/* The same transpose on device memory (no reference counterpart): n_records
 * records of n_bits bits, each padded to 16 bits, into n_bits records of
 * n_records bits padded to 16 bits, enqueued on `stream` (NULL: the library
 * stream).  Returns 0, or -1 on bad arguments. */
int lakgb_bits_transpose_device(const unsigned char *in, int n_records, int n_bits, unsigned char *out,
                                void *stream);

/* Grouped Gram (no reference counterpart): n independent Grams, each as
 * lakgb_gram_device would compute it (bit-identical outputs), run as ONE
 * persistent launch of the tensor-core kernel over all their tiles (plus one
 * launch that builds every instance's block tables) -- for many instances at
 * once, e.g. the Gram passes of label-shuffled null problems.  create copies
 * the descriptors to the device (the pointers in them must stay valid; the
 * data they point to may change between runs); run enqueues the two launches
 * on `stream` (NULL: the library stream) and does nothing else, so it can be
 * captured in a CUDA graph.  All instances must have the same type_flag; a
 * symmetric instance must have as many 128-row tiles of A rows as of Z rows.
 * create returns NULL on bad arguments (lakgb_last_error says why). */
typedef struct lakgb_gram_group lakgb_gram_group;
lakgb_gram_group *lakgb_gram_group_create(const struct lakgb_gram_args *args, int n);
int lakgb_gram_group_run(lakgb_gram_group *group, void *stream);
void lakgb_gram_group_destroy(lakgb_gram_group *group);

/* Device mirrors of L_handles (no reference counterpart).  After
 * lakgb_L_mirror(L) the values of L live on the device: the kernel entry
 * points above write a mirrored output there (not into L->lf) and read a
 * mirrored input from there; lakgb_L_to_host copies them back into L->lf.
 * lakgb_L_sub (dst->lf[i] -= src->lf[i] for i < dst->length) and
 * lakgb_L_transpose (L2_transpose, dir_c/L_init.c:31-38) run on the device
 * when both handles are mirrored.  The bcc solve mirrors its Gram matrices
 * (AnZt, AnAt and their low-rank updates) for the whole solve. */
void lakgb_L_mirror(struct L_handle *L);
/* lakgb_L_mirror for an L whose values are all zero (e.g. just allocated):
 * the device copy is zero-filled instead of uploaded. */
void lakgb_L_mirror_zero(struct L_handle *L);
void lakgb_L_release_mirror(struct L_handle *L);
void lakgb_L_to_host(struct L_handle *L);
void lakgb_L_sub(struct L_handle *dst, const struct L_handle *src);
void lakgb_L_transpose(struct L_handle *dst, const struct L_handle *src);

/* Joined groups of calls (the reference runs a stage's calls on thread slots
 * and joins them with GLOBAL_pthread_tuc): between lakgb_defer_begin and the
 * matching lakgb_defer_end, this host thread's calls write their host
 * outputs only when the outermost scope ends -- the kernels are enqueued and
 * the copies into the L_handles made then, with one wait for all of them.
 * wrap_AnZt_S_WnYt_vv__run, wrap_AtTYn____WtSZn_vv__run and (with residency
 * on and the tensor-core bit-plane kernel, B_MLT 8 / 16 / 32)
 * wrap_At_T_YnWt_S_Zn_ww__run calls are also held back and run as one
 * launch per entry point then (their FP64 sums are long dependent chains).
 * Read the outputs only after lakgb_defer_end; every output equals the one
 * the call makes alone. */
void lakgb_defer_begin(void);
void lakgb_defer_end(void);

/* Allocation-free quantisation (no counterpart in the reference): the
 * arithmetic of wrap_xcalc on caller-owned device buffers, for callers that
 * must not allocate device memory -- e.g. a process whose device memory is
 * fully reserved up front by its own pool (the serving loop admits solves by
 * HBM footprint), or code on a path where a cudaMalloc would synchronise the
 * device.  Its scratch is one static device array of
 * 3 * LAKGB_XCALC_NOALLOC_MAX_COLS + 4 doubles (786,464 bytes), so at most
 * LAKGB_XCALC_NOALLOC_MAX_COLS retained columns; larger problems are rejected
 * with an error.  The array is shared by every call on a device: calls whose
 * kernels overlap on the GPU race.  The first call on a device looks the array
 * up (cudaGetSymbolAddress) and should come before any stream capture.
 * The call is synchronous: it returns once its GPU work is done (it reads
 * {min, max, mlt} back into host memory).
 * Inputs (device): lf, the element offset of each Yn a-row (-1 = not
 * retained, nrows_a entries), of each retained row (rows_j) and column
 * (cols_j) in j order, and plane 0 (row0, brows bytes, may be NULL).
 * Output: planes ((b_mlt+1)*n_cols_j rows of brows bytes, overwritten) and,
 * in host memory, {min, max, mlt} as wrap_xcalc stores them in M_X.
 * Requirements: planes 4-byte aligned; brows a multiple of 4 and at least
 * 4*ceil(nrows_a/32) (wrap_xcalc's plane rows, bsize(nrows_a) bytes, are);
 * counts >= 0; 1 <= b_mlt <= 62; d_mlt >= 2.  Returns 0, or non-zero with
 * lakgb_last_error() set and nothing launched. */
#define LAKGB_XCALC_NOALLOC_MAX_COLS 32768
struct lakgb_xcalc_noalloc_args {
  const double *lf;
  const long long *row_off_a; int nrows_a;
  const long long *rows_j; int n_rows_j;
  const long long *cols_j; int n_cols_j;
  const unsigned char *row0;
  int b_mlt; long long d_mlt; long long brows;
  unsigned char *planes;
  double *min_max_mlt;
  void *stream;   /* cudaStream_t; NULL = the legacy default stream */
};
int lakgb_xcalc_noalloc(const struct lakgb_xcalc_noalloc_args *args);

/* ---------------------------------------------------------------------------
 * Library control (no reference counterpart).
 * ------------------------------------------------------------------------- */

/* Last error recorded by any entry point (0 = none) and its message; reading
 * it clears it. */
int lakgb_last_error(char *msg, int msg_len);
/* The first error recorded by entry points called on this thread since the
 * previous call (0: none), with its message; clears it.  Each thread keeps its
 * own, so concurrent callers (one solve per thread) see only theirs; the
 * whole-solve entry points check it and fail with code 9 when a kernel entry
 * point they called reported an error. */
int lakgb_thread_error_take(char *msg, int msg_len);
/* Keep uploaded wX bit matrices resident on the device between calls, keyed
 * by their host address and size (1), or upload them afresh on every call (0,
 * default).  With 1, a caller that rewrites a wX buffer in place, or frees one
 * whose address may be reused, must call lakgb_forget_host_buffer first.
 * lakgb_bcc_solve and lakgb_bcc_run_in_file keep their own matrices resident
 * for the length of the solve whatever this setting is. */
void lakgb_set_residency(int on);
void lakgb_forget_host_buffer(const void *host_ptr);
/* D_MLT used by wrap_xcalc (the reference's GLOBAL_D_MLT, default 2^32). */
void lakgb_set_d_mlt(long long d_mlt);
/* Number of CUDA kernels this library has launched since load. */
unsigned long long lakgb_kernel_launches(void);
/* Device time (ms) of the most recent Gram kernel launch, timed with CUDA
 * events on the launching stream. */
double lakgb_last_gram_ms(void);
/* Per-entry-point call counts and wall seconds (host clock, each call's own
 * synchronisations included) as JSON, collected only when the environment
 * sets LAKGB_PROFILE_CALLS; returns the full length.  Reset clears them. */
int lakgb_call_profile(char *buf, int buf_len);
void lakgb_call_profile_reset(void);
/* Kernel of the +/-1 Gram (AnZt_vv / AnAt_vv and the Grams inside the bcc
 * solve): LAKGB_GRAM_TENSOR runs the integer counts on the tcgen05 tensor
 * cores, LAKGB_GRAM_POPCOUNT on the CUDA cores' popcount, LAKGB_GRAM_AUTO
 * (default) chooses per shape class by measurement; all give bit-identical
 * outputs.  Process-wide. */
#define LAKGB_IMPL_POPCOUNT 0
#define LAKGB_IMPL_TENSOR 1
#define LAKGB_IMPL_AUTO 2
/* Gram only: the popcount kernel split over blocks (every 1920-column block
 * of every output tile counted by its own CTA, then the FP64 fold over the
 * blocks in order); for launches with few output tiles.  Bit-identical. */
#define LAKGB_IMPL_SPLIT 3
#define LAKGB_GRAM_POPCOUNT LAKGB_IMPL_POPCOUNT
#define LAKGB_GRAM_TENSOR LAKGB_IMPL_TENSOR
#define LAKGB_GRAM_AUTO LAKGB_IMPL_AUTO
void lakgb_set_gram_impl(int impl);
int lakgb_gram_impl(void);
/* LAKGB_GRAM_AUTO (the default) picks the Gram kernel and tile shape by
 * measurement: the first launch of each shape class (type, symmetric, log2 of
 * the A rows, Z rows and blocks) runs every candidate -- the tensor-core
 * kernel, two tile shapes of the popcount kernel and the popcount kernel
 * split over blocks, all bit-identical --
 * timed with CUDA events, and the fastest serves that class afterwards.
 * lakgb_gram_autotune_table writes the table as JSON into buf (returns its
 * full length); lakgb_gram_autotune_reset clears it. */
int lakgb_gram_autotune_table(char *buf, int buf_len);
void lakgb_gram_autotune_reset(void);
/* Kernel of the bit-plane loop product (wrap_At_T_YnWt_S_Zn_ww__run):
 * LAKGB_IMPL_TENSOR (default; B_MLT of 8, 16 or 32, otherwise the CUDA-core
 * kernel runs) or LAKGB_IMPL_POPCOUNT; bit-identical outputs.  Process-wide. */
void lakgb_set_bitplane_impl(int impl);
int lakgb_bitplane_impl(void);
/* Device status word of the tensor-core kernels: 0, or the code of the first
 * pipeline wait that ran out of time (the kernel then skipped its remaining
 * work, so its outputs are invalid).  Synchronises the device; reading it
 * clears it. */
int lakgb_device_status(void);
/* The same status word, but only the calling thread's own: every host thread
 * has its own word, written by the tensor-core launches it makes.  Waits for
 * the thread's own stream (not the device); reading clears it.  A whole solve
 * (lakgb_bcc_solve) checks it on return and fails if it is set. */
int lakgb_thread_device_status(void);
/* Test hook of the tensor-core Gram's bounded waits (no reference
 * counterpart): wall-time limit of one pipeline wait in ns (0 = the default,
 * 2 s) and, when `withhold` is non-zero, one producer arrival of the first
 * operand stage of CTA 0 is withheld in every later Gram launch, so that the
 * MMA warp's wait runs out: the kernel then skips its remaining work, frees
 * its tensor memory and returns, and the status word reads 4.  Synchronises
 * the device. */
void lakgb_debug_tc_pipeline(unsigned long long wait_limit_ns, int withhold);
/* Measured FP64 add throughput of the current device (adds per second):
 * independent add chains on every SM, best of three timed launches.  The fold
 * of the tensor-core Gram performs one FP64 add per output element per
 * 1920-column block, so this rate bounds it. */
double lakgb_measure_fp64_add_rate(void);

#ifdef __cplusplus
}
#endif
#endif /* LAKCLUSTER_GB300_H */
