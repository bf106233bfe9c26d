/* lak_oracle_wrap.c -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's wrap_* entry points (signatures of
 * include/lakcluster_gb300.h) implemented by the plain-C restatement in
 * lak_oracle.c, so that the package's solve driver can be linked against the
 * oracle (oracle/lakbcc_port): a whole bcc solve on the host cores that
 * builds on every machine, used as the CPU baseline where the reference
 * itself cannot be compiled (it needs x86 SSE2) and as a second, independent
 * check of the GPU library's whole-solve outputs.  The thread-slot arguments
 * are ignored; each call runs to completion (OpenMP inside). */
#include "lak_oracle.h"

int wrap_AnZt_vv__run(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, int sc,
                      struct M_handle *M_An, struct M_handle *M_Zn, double *A_ajdk,
                      struct L_handle *lfA, struct L_handle *lfZ, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AnZt_vv(type_flag, sr, sc, M_An, M_Zn, A_ajdk, lfA, lfZ, out);
}

int wrap_AnAt_vv__run(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, int sc,
                      struct M_handle *M_An, struct M_handle *M_Zn, double *A_ajdk,
                      struct L_handle *lfA, struct L_handle *lfZ, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AnAt_vv(type_flag, sr, sc, M_An, M_Zn, A_ajdk, lfA, lfZ, out);
}

int wrap_An_v__run(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, struct M_handle *M_An,
                   struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_An_v(type_flag, sr, M_An, out);
}

int wrap_An_ajdk_v(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, struct M_handle *M_An,
                   double *A_ajdk, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_An_ajdk_v(type_flag, sr, M_An, A_ajdk, out);
}

void wrap_xcalc(int *tidx, void **vpra, pthread_t *th, unsigned char *mr_j, unsigned char *mr_b,
                unsigned char *mc_j, unsigned char *mc_b, struct L_handle *lf, double *YnWt, int *Yn_nrows_p,
                int *Wn_nrows_p, struct M_handle **M_X_p, int *b_mlt_p, int trm_flag)
{
  (void)tidx; (void)vpra; (void)th;
  lako_xcalc(mr_j, mr_b, mc_j, mc_b, lf, YnWt, *Yn_nrows_p, *Wn_nrows_p, *M_X_p, *b_mlt_p, trm_flag);
}

int wrap_At_T_YnWt_S_Zn_ww__run(int *tidx, void **vpra, pthread_t *th, int sa, int st, struct M_handle *M_At,
                                struct M_handle *M_Tt, struct M_handle *M_Yn, struct M_handle *M_Wn,
                                struct M_handle *M_St, struct M_handle *M_Zt, double *A_ajdk,
                                struct M_handle *M_YnWt, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_At_T_YnWt_S_Zn_ww(sa, st, M_At, M_Tt, M_Yn, M_Wn, M_St, M_Zt, A_ajdk, M_YnWt, out);
}

int wrap_AnZt_S_WnYt_vv__run(int *tidx, void **vpra, pthread_t *th, int sa, int ss, struct M_handle *M_An,
                             struct M_handle *M_St, struct M_handle *M_Zn, struct L_handle *lf_AnZt,
                             struct L_handle *lf_YnWt, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AnZt_S_WnYt_vv(sa, ss, M_An, M_St, M_Zn, lf_AnZt, lf_YnWt, out);
}

int wrap_An_ZtSn_ww__run(int *tidx, void **vpra, pthread_t *th, int sa, int ss, struct M_handle *M_An,
                         struct L_handle *lf_ZtSn, struct M_handle *M_ZtSn, struct M_handle *M_St,
                         struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th; (void)lf_ZtSn;
  return lako_An_ZtSn_ww(sa, ss, M_An, M_ZtSn, M_St, out);
}

int wrap_AtTYn_vv__run(int *tidx, void **vpra, pthread_t *th, int sa, int sy, int st, struct M_handle *M_At,
                       struct M_handle *M_Tt, struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk,
                       struct L_handle *lf_AtTn, struct L_handle *lf_YtTn, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AtTYn_vv(sa, sy, st, M_At, M_Tt, M_Yt, A_ajdk, Y_ajdk, lf_AtTn, lf_YtTn, out);
}

int wrap_AtTYn____WtSZn_vv__run(int *tidx, void **vpra, pthread_t *th, int sa, int ss, struct M_handle *M_At,
                                struct M_handle *M_Tt, struct M_handle *M_Yt, struct M_handle *M_Wt,
                                struct M_handle *M_St, struct M_handle *M_Zt, double *Y_ajdk,
                                struct L_handle *lf_AtTYn, struct L_handle *lf_ZtSWn, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AtTYn____WtSZn_vv(sa, ss, M_At, M_Tt, M_Yt, M_Wt, M_St, M_Zt, Y_ajdk, lf_AtTYn, lf_ZtSWn, out);
}

int wrap_AtTAn_vv__run(int *tidx, void **vpra, pthread_t *th, int sa, int sy, int st, struct M_handle *M_At,
                       struct M_handle *M_Tt, struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk,
                       struct L_handle *lf_AtTn, struct L_handle *lf_YtTn, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AtTAn_vv(sa, sy, st, M_At, M_Tt, M_Yt, A_ajdk, Y_ajdk, lf_AtTn, lf_YtTn, out);
}

int wrap_M_At_to_L2_run(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, int sc, struct M_handle *M_At,
                        double *A_ajdk, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_M_to_L2(1, type_flag, sr, sc, M_At, A_ajdk, out);
}

int wrap_M_An_to_L2_run(int *tidx, void **vpra, pthread_t *th, int type_flag, int sr, int sc, struct M_handle *M_An,
                        double *A_ajdk, struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_M_to_L2(0, type_flag, sr, sc, M_An, A_ajdk, out);
}

int wrap_AnZt_mm__run(int *tidx, void **vpra, pthread_t *th, struct L_handle *lf_At, struct L_handle *lf_Zt,
                      struct L_handle **out)
{
  (void)tidx; (void)vpra; (void)th;
  return lako_AnZt_mm(lf_At, lf_Zt, out);
}
