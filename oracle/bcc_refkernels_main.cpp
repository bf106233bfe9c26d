// Test infrastructure: the package's bcc solve driver (lakcluster_c_gb300/csrc
// bcc_driver.cpp) linked against the reference's own wrap_* kernels in
// _ref/liblakref.so instead of the GPU library.  Comparing its trace with the
// reference program's (_ref/lakcluster_ref) on the same .in file checks the
// driver's host logic with the kernels held fixed; comparing it with the GPU
// build checks the kernels with the driver held fixed.
//
// usage: lakbcc_refkernels file.in      (writes out_trace.txt / out_xdrop_*.txt
//                                        into the .in file's GLOBAL_DIR_NAME)
#include <dlfcn.h>
#include <stdio.h>

#include "../lakcluster_c_gb300/csrc/bcc_driver.h"

// The reference program reads one 1920-bit block past the end of zero-length
// buffers when it sums the columns of an empty control matrix (An_v on M_Zt
// with Z_nrows = 0, dir_c/bcc.c:1228 -> An_v.c:49 -> popcount.c:46-69: the SSE
// loop is a do-while).  What it reads is the allocator's bookkeeping next to
// those buffers, so every SNP's combined count picks up a small layout-
// dependent constant.  When LAKREF_EMPTY_Z_ROWSUM is set, this harness adds
// that constant (measured from the reference program's AZ_rsum.mda) to the
// same An_v call, so that the rest of the solve can be compared bit for bit.
extern "C" int wrap_An_v__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                              int output_spacing_r, struct M_handle *M_An,
                              struct L_handle **output_An_v_p) {
  typedef int (*fn_t)(int *, void **, pthread_t *, int, int, struct M_handle *, struct L_handle **);
  static fn_t real = (fn_t)dlsym(RTLD_NEXT, "wrap_An_v__run");
  const int rc = real(tidx, vpra, thread_in, type_flag, output_spacing_r, M_An, output_An_v_p);
  const char *bias = getenv("LAKREF_EMPTY_Z_ROWSUM");
  if (bias && type_flag == LAKGB_TYPE_00 && M_An->ncols == 0 && output_spacing_r == LAKGB_SPACING_a) {
    const double b = atof(bias);
    for (long long j = 0; j < M_An->rpop_j; ++j) (*output_An_v_p)->lf[M_An->m_a_[j]] += b;
  }
  return rc;
}

extern "C" {
int lakref_init(long long mb, int nthreads, int omp_on);
extern long long GLOBAL_D_MLT;
extern int GLOBAL_B_MLT;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s file.in\n", argv[0]);
    return 2;
  }
  lakbcc::Params P;
  lakbcc::Input I;
  lakbcc::Output O;
  std::string err;
  int rc = lakbcc::read_in_file(argv[1], P, I, err);
  if (rc) { fprintf(stderr, "error: %s\n", err.c_str()); return rc; }
  const char *mb = getenv("LAKREF_MB");
  if (lakref_init(mb ? atoll(mb) : 4096, 1, 0)) { fprintf(stderr, "error: arena\n"); return 1; }
  GLOBAL_D_MLT = P.D_MLT;
  GLOBAL_B_MLT = P.B_MLT;
  if (P.test_type == "lakcluster_scorebox" || P.test_type == "dexcluster_scorebox") {
    lakbcc::ScoreboxOutput SO;
    rc = lakbcc::scorebox(P, I, SO, err);
    if (rc) { fprintf(stderr, "error: %s\n", err.c_str()); return rc; }
    if (lakbcc::make_output_dir(P.dir_name) || lakbcc::write_scorebox(P.dir_name, SO)) {
      fprintf(stderr, "error: cannot write outputs into %s\n", P.dir_name.c_str());
      return 2;
    }
    return 0;
  }
  rc = P.test_type == "dexcluster_driver" ? lakbcc::dcc_solve(P, I, O, err) : lakbcc::solve(P, I, O, err);
  if (rc) { fprintf(stderr, "error: %s\n", err.c_str()); return rc; }
  if (lakbcc::make_output_dir(P.dir_name) || lakbcc::write_outputs(P.dir_name, O)) {
    fprintf(stderr, "error: cannot write outputs into %s\n", P.dir_name.c_str());
    return 2;
  }
  return 0;
}
