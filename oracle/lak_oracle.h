/* lak_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's bcc kernels, used as the checker
 * for the GPU library (tests/, __graft_entry__.smoke) and as the CPU baseline
 * timed by bench.py.  Nothing in the product links or calls it.
 *
 * Each function follows the reference routine cited beside it, on the same
 * M_handle / L_handle structs, without the thread-slot arguments.  The oracle
 * is pinned against the reference itself: tests/golden/ holds outputs of the
 * reference's own wrap_* kernels (compiled from its sources by
 * oracle/Makefile) on seeded inputs, and tests/test_oracle_golden.py checks
 * this restatement against them bit for bit.
 */
#ifndef LAK_ORACLE_H
#define LAK_ORACLE_H
#include "../include/lakcluster_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* dir_c/AnZt_vv.c:5-223 (get_AnZt_vv__run / wrap_AnZt_vv__run) */
int lako_AnZt_vv(int type_flag, int spacing_r, int spacing_c, struct M_handle *M_An,
                 struct M_handle *M_Zn, double *A_ajdk, struct L_handle *lf_An_ajdk,
                 struct L_handle *lf_Zn_ajdk, struct L_handle **out_p);
/* dir_c/AnAt_vv.c:5-190 (get_AnAt_vv__run / wrap_AnAt_vv__run) */
int lako_AnAt_vv(int type_flag, int spacing_r, int spacing_c, struct M_handle *M_An,
                 struct M_handle *M_Zn, double *A_ajdk, struct L_handle *lf_An_ajdk,
                 struct L_handle *lf_Zn_ajdk, struct L_handle **out_p);
/* dir_c/An_v.c:5-84 */
int lako_An_v(int type_flag, int spacing_r, struct M_handle *M_An, struct L_handle **out_p);
/* dir_c/An_ajdk_v.c:272-388 */
int lako_An_ajdk_v(int type_flag, int spacing_r, struct M_handle *M_An, double *A_ajdk,
                   struct L_handle **out_p);
/* dir_c/An_ajdk_v.c:5-30 */
void lako_calc_A_ajdk(const double *A_p, int A_pcols, double *A_ajdk);

/* dir_c/xcalc.c:5-246 (into a pre-allocated M_X; D_MLT from lako_set_d_mlt) */
void lako_xcalc(unsigned char *mr_j, unsigned char *mr_b, unsigned char *mc_j, unsigned char *mc_b,
                struct L_handle *lf_YnWt, double *YnWt, int Yn_nrows, int Wn_nrows, struct M_handle *M_X,
                int b_mlt, int trm_flag);
void lako_set_d_mlt(long long d_mlt);
/* dir_c/At_T_YnWt_S_Zn_ww.c:5-190 */
int lako_At_T_YnWt_S_Zn_ww(int spacing_a, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_Yn, struct M_handle *M_Wn, struct M_handle *M_St,
                           struct M_handle *M_Zt, double *A_ajdk, struct M_handle *M_YnWt,
                           struct L_handle **out_p);
/* dir_c/An_ZtSWn_Yt_ww.c:5-111 */
int lako_An_ZtSWn_Yt_ww(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle **M_ZtSWn_, struct M_handle *M_Wt, struct M_handle *M_Yn,
                        double *A_ajdk, double *Y_ajdk, struct L_handle **out_p);
/* dir_c/An_ZtSn_ww.c:5-136 */
int lako_An_ZtSn_ww(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_ZtSn,
                    struct M_handle *M_St, struct L_handle **out_p);
/* dir_c/AnZt_S_WnYt_vv.c:5-101 */
int lako_AnZt_S_WnYt_vv(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle *M_Zn, struct L_handle *lf_AnZt, struct L_handle *lf_YnWt,
                        struct L_handle **out_p);
/* dir_c/AtTYn_vv.c:5-202 */
int lako_AtTYn_vv(int spacing_a, int spacing_y, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                  struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_AtTn,
                  struct L_handle *lf_YtTn, struct L_handle **out_p);
/* dir_c/AtTYn____WtSZn_vv.c:5-115 */
int lako_AtTYn____WtSZn_vv(int spacing_a, int spacing_s, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_Yt, struct M_handle *M_Wt, struct M_handle *M_St,
                           struct M_handle *M_Zt, double *Y_ajdk, struct L_handle *lf_AtTYn,
                           struct L_handle *lf_ZtSWn, struct L_handle **out_p);

/* dir_c/AtTAn_vv.c:5-172 */
int lako_AtTAn_vv(int spacing_a, int spacing_y, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                  struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_AtTn,
                  struct L_handle *lf_YtTn, struct L_handle **out_p);
/* dir_c/At_T_YnWt_S_Zn_vv.c:5-85 */
int lako_At_T_YnWt_S_Zn_vv(int spacing_a, int spacing_s, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_St, struct M_handle *M_Zt, double *A_ajdk,
                           struct L_handle *lf_YnWt, struct L_handle **out_p);
/* dir_c/An_ZtSWn_Yt_vv.c:5-130 */
int lako_An_ZtSWn_Yt_vv(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle *M_Yn, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_ZtSWn,
                        struct L_handle **out_p);

/* dir_c/M_Ax_to_L2.c:5-100 (at = 0) and :137-280 (at = 1) */
int lako_M_to_L2(int at, int type_flag, int spacing_r, int spacing_c, struct M_handle *M, double *A_ajdk,
                 struct L_handle **out_p);
/* dir_c/AnZt_mm.c:6-109 (GSL CBLAS dgemm order: ascending k from +0) */
int lako_AnZt_mm(struct L_handle *lf_At, struct L_handle *lf_Zt, struct L_handle **out_p);

/* dir_c/binary_read.c:174-269 (wrap_transpose), on memory: n_in_rec records
 * of in_rec_bytes bytes (bits MSB first) into n_out_rec records of
 * out_rec_bytes bytes, out record r bit c = in record c bit r; bits of out
 * records past the last input record are zero. */
void lako_bits_transpose(const unsigned char *in, long long in_rec_bytes, int n_in_rec, unsigned char *out,
                         long long out_rec_bytes, int n_out_rec);

/* Threads used by the OpenMP loops (default: all). */
void lako_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
