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

/* Threads used by the OpenMP loops (default: all). */
void lako_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
