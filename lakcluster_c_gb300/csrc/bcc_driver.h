// The bcc solve (lakcluster_driver, dir_c/lakcluster_driver.c:14-251) for the
// YnWt row/column strategies, driving the reference-compatible kernel entry
// points.  Internal header shared by the driver translation units.
#pragma once
#include <string>
#include <vector>

#include "bcc_model.h"

namespace lakbcc {

// Solve parameters (the reference's GLOBAL_* settings used on this path).
struct Params {
  int nbins = 1;
  int B_MLT = 32;
  long long D_MLT = 4294967296LL;
  double gamma = 0.125;
  int gamma_type = 0;          // GLOBAL_gamma__log
  int Ireq = 0;
  int test_sparse = 1;         // GLOBAL_TEST_sparse: 0 fixes every allele frequency at 0.5
  double kappa_squared = 0.0;
  double tolerance = 0.000000000001;
  unsigned recursion_limit = 1024 * 32;
  std::string QR_strategy = "YnWt", QC_strategy = "YnWt";
  std::string dir_name;        // output directory (GLOBAL_DIR_NAME); empty: no files
  // GLOBAL_TEST_TYPE: lakcluster_driver (the solve) or lakcluster_scorebox
  std::string test_type = "lakcluster_driver";
  // scorebox grid (GLOBAL_scorebox_row_max / _row_num / _col_max / _col_num)
  int scorebox_row_max = 0, scorebox_row_num = 0, scorebox_col_max = 0, scorebox_col_num = 0;
  // bed_to_b16 (GLOBAL_fname_{bed,bim,fam}_0in, GLOBAL_fname_{b16,bim,fam}_out
  // and the four thresholds, defaults as dir_c/lakcluster_ver18.c:150-163)
  struct BedFiles {
    std::string bed, bim, fam, b16_out, bim_out, fam_out;
    double snp_mss = 0.01, snp_maf = 0.25, snp_I_opt = 0.01, pat_mss = 0.04;
    // b16_merge: GLOBAL_n_file studies GLOBAL_fname_{b16,bim,fam}_0in_
    int n_file = 0;
    std::vector<std::string> b16_in, bim_in, fam_in;
  } bed;
};

// One bin's inputs: packed rows of A (patients x SNPs, bsize(ncols) bytes per
// row, all rows in a-space), the row mask (null: all rows), same for Z.
struct BinInput {
  int A_nrows = 0, Z_nrows = 0;
  std::vector<unsigned char> A_rows, Z_rows;   // a-space rows, bsize(ncols) bytes each
  std::vector<unsigned char> A_mr_b, Z_mr_b;   // bsize(nrows) bytes; empty = all on
  // covariates: T (cases x T_ncols) and S (controls x T_ncols), a-space rows of
  // bsize(T_ncols) bytes; empty = the reference's default single column of
  // ones (T_ncols must then be 1)
  std::vector<unsigned char> T_rows, S_rows;
};

struct Input {
  // out_xdrop lines of earlier runs as (row, column) pairs, -1 where absent:
  // the scorebox order (GLOBAL_scorebox_out_xdrop) and the scrambles applied
  // after loading (GLOBAL_scramble_out_xdrop_ / GLOBAL_scramble_rseed_)
  std::vector<int> scorebox_xdrop;
  struct Scramble {
    std::vector<int> xdrop;
    unsigned long long rseed = 1;
  };
  std::vector<Scramble> scramble;
  int ncols = 0;
  int T_ncols = 1;                             // covariate columns (GLOBAL_T_n_cols)
  std::vector<unsigned char> mc_b;             // bsize(ncols) bytes; empty = all on
  std::vector<BinInput> bins;
};

struct Output {
  std::vector<int> xdrop_a, xdrop_b;          // pairs (row, col)
  std::vector<double> trace;                  // 6 values per iteration
  int iterations = 0;
  // further files the reference writes into the output directory: the case
  // rows before and after a scramble (*_scramble_pre.b16 / _pos.b16), as
  // (file name, contents)
  std::vector<std::pair<std::string, std::vector<unsigned char>>> files;
};

// Callbacks into the kernel library that owns the entry points the solve
// calls: release an output L_handle the library allocated, and drop any
// device copy cached for a host buffer that is about to be freed.  Either may
// be null (nothing to release).
struct Hooks {
  void (*release_L)(L_handle *L) = nullptr;
  void (*forget_host)(const void *p) = nullptr;
  // Device mirrors for the large score matrices (AnZt, AnAt and their
  // low-rank updates): keep L's values on the device, drop the mirror, copy
  // the device values back into L->lf, and the two matrix operations the
  // driver applies to them (dst -= src elementwise; L2_transpose).  All null:
  // the matrices stay on the host.
  void (*L_mirror)(L_handle *L) = nullptr;
  void (*L_release_mirror)(L_handle *L) = nullptr;
  void (*L_to_host)(L_handle *L) = nullptr;
  void (*L_sub)(L_handle *dst, const L_handle *src) = nullptr;
  void (*L_transpose)(L_handle *dst, const L_handle *src) = nullptr;
  // As L_mirror for an L whose values are all zero (freshly allocated): the
  // device copy is zero-filled, nothing is uploaded.  Null: L_mirror is used.
  void (*L_mirror_zero)(L_handle *L) = nullptr;
  // A scope whose kernel calls may run together when it ends (the reference
  // runs them on thread slots and joins them, GLOBAL_pthread_tuc): outputs
  // are read only after defer_end.  Null: every call completes at once.
  void (*defer_begin)() = nullptr;
  void (*defer_end)() = nullptr;
};

// The scorebox grid (S_handle outputs, dir_c/S_init.c): row_num x col_num
// arrays, row index fastest.
struct ScoreboxOutput {
  int row_max = 0, row_num = 0, col_max = 0, col_num = 0;
  std::vector<int> A_rpop_j_total, A_cpop_j, Irem;
  std::vector<double> QR_avg, QC_avg;
};

// Parse a reference .in file (updateglobals.c syntax) and load its .b16 files.
int read_in_file(const char *path, Params &P, Input &I, std::string &err);
// Create the output directory when it does not exist (set_globals,
// lakcluster_ver18.c:231).
int make_output_dir(const std::string &dir);
// Run the solve.  Returns 0 on success.
int solve(const Params &P, const Input &I, Output &O, std::string &err, const Hooks *hooks = nullptr);
// Run the dexcluster method (GLOBAL_TEST_TYPE dexcluster_driver) instead.
int dcc_solve(const Params &P, const Input &I, Output &O, std::string &err, const Hooks *hooks = nullptr);
// Run the scorebox (GLOBAL_TEST_TYPE lakcluster_scorebox) over I.scorebox_xdrop.
int scorebox(const Params &P, const Input &I, ScoreboxOutput &SO, std::string &err, const Hooks *hooks = nullptr);
// Write its five .mda arrays into dir (names as S_handle_dmp writes them).
int write_scorebox(const std::string &dir, const ScoreboxOutput &SO);
// A check the solves of the calling thread run before the initial pass and
// before every elimination iteration: a non-zero return ends the solve with
// that code (its buffers released as on any return) and `why` as the error.
// Null clears it.  Used by the serving loop for cancellation and deadlines.
using StopCheck = int (*)(void *ctx, const char **why);
void set_stop_check(StopCheck fn, void *ctx);
// Write out_trace.txt / out_xdrop_a.txt / out_xdrop_b.txt as the reference does.
int write_outputs(const std::string &dir, const Output &O);

}  // namespace lakbcc
