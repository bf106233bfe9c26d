// C entry points for a whole bcc solve on the GPU library: the .in-file
// program (the reference's main -> read_input -> lakcluster_driver,
// dir_c/lakcluster_ver18.c:238-330 and dir_c/lakcluster_driver.c:14-251) and
// an in-memory variant for callers that hold the packed matrices already.
#include <stdlib.h>
#include <string.h>

#include <string>

#include "bcc_driver.h"

#include "../../include/lakcluster_gb300.h"

namespace {

thread_local std::string g_err;

void release_L(L_handle *L) {
  if (!L) return;
  free(L->lf);
  free(L);
}

const lakbcc::Hooks kHooks = {release_L,       lakgb_forget_host_buffer, lakgb_L_mirror,      lakgb_L_release_mirror,
                               lakgb_L_to_host, lakgb_L_sub,              lakgb_L_transpose, lakgb_L_mirror_zero,
                               lakgb_defer_begin, lakgb_defer_end};

long row_bytes_min(int ncols) { return (long)(ncols + (16 - ncols % 16) % 16) / 8; }

// A tensor-core pipeline wait of this thread's launches that ran out of time
// invalidates the solve's products: report it as the solve's error.
int pipeline_status() {
  const int st = lakgb_thread_device_status();
  char msg[256];
  const int e = lakgb_thread_error_take(msg, sizeof msg);
  if (st) {
    g_err = "a tensor-core pipeline wait ran out of time (code " + std::to_string(st) + "); results invalid";
    return 8;
  }
  if (e) {
    g_err = std::string("a kernel entry point failed: ") + msg;
    return 9;
  }
  return 0;
}

// Forget this thread's leftovers from earlier calls before a solve starts.
void pipeline_reset() {
  lakgb_thread_device_status();
  lakgb_thread_error_take(nullptr, 0);
}

}  // namespace

extern "C" void lakgb_bcc_problem_init(struct lakgb_bcc_problem *p) {
  memset(p, 0, sizeof(*p));
  p->T_ncols = 1;
  p->B_MLT = 32;
  p->gamma = 0.125;
  p->gamma_type = 0;
  p->test_sparse = 1;
}

extern "C" void lakgb_residency_scope(int enter);   // lakgb_runtime.cu
extern "C" void lakgb_device_only_planes(int on);   // lakgb_runtime.cu

namespace {
// Device residency of the solve's matrices for the length of one solve: the
// driver forgets each buffer it frees or rewrites, and whatever is still
// cached when the solve ends is dropped.  Unless the solve traces its stages
// (LAKBCC_TRACE, which digests bit planes on the host), xcalc's planes stay on
// the device.
struct SolveResidency {
  SolveResidency() {
    lakgb_residency_scope(1);
    const char *trace = getenv("LAKBCC_TRACE");
    lakgb_device_only_planes(!(trace && *trace));
  }
  ~SolveResidency() {
    lakgb_device_only_planes(0);
    lakgb_residency_scope(0);
  }
};
}  // namespace

extern "C" int lakgb_bcc_solve(const struct lakgb_bcc_problem *prob, struct lakgb_bcc_result *res) {
  SolveResidency residency;
  g_err.clear();
  pipeline_reset();
  if (!prob || !res) { g_err = "null argument"; return 2; }
  memset(res, 0, sizeof(*res));
  if (prob->nbins <= 0 || !prob->bins || prob->ncols < 0) { g_err = "bad problem description"; return 2; }
  if (prob->row_bytes < row_bytes_min(prob->ncols)) { g_err = "row_bytes smaller than one packed row"; return 2; }
  lakbcc::Params P;
  P.nbins = prob->nbins;
  P.B_MLT = prob->B_MLT;
  P.D_MLT = 1LL << prob->B_MLT;
  P.gamma = prob->gamma;
  P.gamma_type = prob->gamma_type;
  P.test_sparse = prob->test_sparse;
  P.Ireq = prob->Ireq;
  P.kappa_squared = prob->kappa_squared;
  if (prob->QC_strategy) P.QC_strategy = prob->QC_strategy;
  if (prob->QR_strategy) P.QR_strategy = prob->QR_strategy;
  lakbcc::Input I;
  I.ncols = prob->ncols;
  I.T_ncols = prob->T_ncols > 0 ? prob->T_ncols : 1;  // 0: the default single column
  const long rb = lakbcc::bsize(prob->ncols), ch = row_bytes_min(prob->ncols);
  if (prob->mc_b) I.mc_b.assign(prob->mc_b, prob->mc_b + ch), I.mc_b.resize(rb, 0);
  I.bins.resize(prob->nbins);
  for (int nb = 0; nb < prob->nbins; ++nb) {
    const struct lakgb_bcc_bin &b = prob->bins[nb];
    lakbcc::BinInput &B = I.bins[nb];
    if (b.A_nrows < 0 || b.Z_nrows < 0 || (b.A_nrows > 0 && !b.A_rows) || (b.Z_nrows > 0 && !b.Z_rows)) {
      g_err = "bad bin description";
      return 2;
    }
    B.A_nrows = b.A_nrows;
    B.Z_nrows = b.Z_nrows;
    B.A_rows.assign((size_t)(b.A_nrows > 0 ? b.A_nrows : 1) * rb, 0);
    for (int r = 0; r < b.A_nrows; ++r) memcpy(&B.A_rows[(size_t)r * rb], b.A_rows + (size_t)r * prob->row_bytes, ch);
    if (b.Z_nrows > 0) {
      B.Z_rows.assign((size_t)b.Z_nrows * rb, 0);
      for (int r = 0; r < b.Z_nrows; ++r) memcpy(&B.Z_rows[(size_t)r * rb], b.Z_rows + (size_t)r * prob->row_bytes, ch);
    }
    if (b.A_mr_b) {
      B.A_mr_b.assign(b.A_mr_b, b.A_mr_b + row_bytes_min(b.A_nrows));
      B.A_mr_b.resize(lakbcc::bsize(b.A_nrows), 0);
    }
    if (b.Z_mr_b) {
      B.Z_mr_b.assign(b.Z_mr_b, b.Z_mr_b + row_bytes_min(b.Z_nrows));
      B.Z_mr_b.resize(lakbcc::bsize(b.Z_nrows), 0);
    }
    // covariate rows, repacked to bsize(T_ncols) bytes per row
    if (!b.T_rows != !b.S_rows || (!b.T_rows && I.T_ncols > 1)) {
      g_err = "covariate rows T_rows and S_rows must be given together (and for T_ncols > 1)";
      return 2;
    }
    if (b.T_rows) {
      const long tch = row_bytes_min(I.T_ncols), tb = lakbcc::bsize(I.T_ncols);
      B.T_rows.assign((size_t)std::max(1, b.A_nrows) * (size_t)tb, 0);
      for (int r = 0; r < b.A_nrows; ++r) memcpy(&B.T_rows[(size_t)r * tb], b.T_rows + (size_t)r * tch, tch);
      B.S_rows.assign((size_t)std::max(1, b.Z_nrows) * (size_t)tb, 0);
      for (int r = 0; r < b.Z_nrows; ++r) memcpy(&B.S_rows[(size_t)r * tb], b.S_rows + (size_t)r * tch, tch);
    }
  }
  lakgb_set_d_mlt(P.D_MLT);
  lakbcc::Output O;
  int rc = lakbcc::solve(P, I, O, g_err, &kHooks);
  if (rc) return rc;
  if ((rc = pipeline_status())) return rc;
  res->iterations = O.iterations;
  res->trace = (double *)malloc(sizeof(double) * (O.trace.size() ? O.trace.size() : 1));
  res->n_xdrop = (int)(O.xdrop_a.size() / 2);
  res->xdrop_a = (int *)malloc(sizeof(int) * (O.xdrop_a.size() ? O.xdrop_a.size() : 1));
  res->xdrop_b = (int *)malloc(sizeof(int) * (O.xdrop_b.size() ? O.xdrop_b.size() : 1));
  if (!res->trace || !res->xdrop_a || !res->xdrop_b) { g_err = "out of host memory"; return 2; }
  if (!O.trace.empty()) memcpy(res->trace, O.trace.data(), sizeof(double) * O.trace.size());
  if (!O.xdrop_a.empty()) memcpy(res->xdrop_a, O.xdrop_a.data(), sizeof(int) * O.xdrop_a.size());
  if (!O.xdrop_b.empty()) memcpy(res->xdrop_b, O.xdrop_b.data(), sizeof(int) * O.xdrop_b.size());
  return 0;
}

extern "C" void lakgb_bcc_result_free(struct lakgb_bcc_result *res) {
  if (!res) return;
  free(res->trace);
  free(res->xdrop_a);
  free(res->xdrop_b);
  memset(res, 0, sizeof(*res));
}

extern "C" int lakgb_bcc_run_in_file(const char *in_path) {
  SolveResidency residency;
  g_err.clear();
  pipeline_reset();
  lakbcc::Params P;
  lakbcc::Input I;
  int rc = lakbcc::read_in_file(in_path, P, I, g_err);
  if (rc) return rc;
  if (P.test_type == "bed_to_b16") {  // lakcluster_ver18.c:361
    struct lakgb_bed_params bp;
    bp.snp_mss_threshold = P.bed.snp_mss; bp.snp_maf_threshold = P.bed.snp_maf;
    bp.snp_I_opt_threshold = P.bed.snp_I_opt; bp.pat_mss_threshold = P.bed.pat_mss;
    rc = lakgb_bed_to_b16(P.bed.bed.c_str(), P.bed.bim.c_str(), P.bed.fam.c_str(), P.bed.b16_out.c_str(),
                          P.bed.bim_out.c_str(), P.bed.fam_out.c_str(), &bp);
    if (rc) {
      char msg[256];
      lakgb_bed_last_error(msg, sizeof msg);
      g_err = msg;
      return rc;
    }
    return pipeline_status();
  }
  if (P.test_type == "b16_merge") {  // lakcluster_ver18.c:364
    std::vector<const char *> b16, bim, fam;
    for (int f = 0; f < P.bed.n_file; ++f) {
      b16.push_back(P.bed.b16_in[f].c_str());
      bim.push_back(P.bed.bim_in[f].c_str());
      fam.push_back(P.bed.fam_in[f].c_str());
    }
    rc = lakgb_b16_merge(P.bed.n_file, b16.data(), bim.data(), fam.data(), P.bed.b16_out.c_str(),
                         P.bed.bim_out.c_str(), P.bed.fam_out.c_str());
    if (rc) {
      char msg[256];
      lakgb_bed_last_error(msg, sizeof msg);
      g_err = msg;
      return rc;
    }
    return pipeline_status();
  }
  lakgb_set_d_mlt(P.D_MLT);
  if (P.test_type == "lakcluster_scorebox" || P.test_type == "dexcluster_scorebox") {  // lakcluster_ver18.c:338
    lakbcc::ScoreboxOutput SO;
    rc = lakbcc::scorebox(P, I, SO, g_err, &kHooks);
    if (rc) return rc;
    if ((rc = pipeline_status())) return rc;
    if (lakbcc::make_output_dir(P.dir_name) || lakbcc::write_scorebox(P.dir_name, SO)) {
      g_err = "cannot write outputs into " + P.dir_name;
      return 2;
    }
    return 0;
  }
  lakbcc::Output O;
  rc = P.test_type == "dexcluster_driver" ? lakbcc::dcc_solve(P, I, O, g_err, &kHooks)  // lakcluster_ver18.c:345
                                          : lakbcc::solve(P, I, O, g_err, &kHooks);
  if (rc) return rc;
  if ((rc = pipeline_status())) return rc;
  if (lakbcc::make_output_dir(P.dir_name) || lakbcc::write_outputs(P.dir_name, O)) {
    g_err = "cannot write outputs into " + P.dir_name;
    return 2;
  }
  return 0;
}

extern "C" int lakgb_bcc_last_error(char *msg, int msg_len) {
  if (msg && msg_len > 0) {
    strncpy(msg, g_err.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return g_err.empty() ? 0 : 1;
}
