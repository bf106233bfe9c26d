// Input side of the bcc solve: the reference's ".in" parameter file
// (read_input / updateglobals, dir_c/updateglobals.c:5-200) and its ".b16"
// bit-matrix files (binary_read, dir_c/binary_read.c:5-37).
//
// A ".in" file is a sequence of "NAME= value;" statements ending with
// "END= 0;".  List-valued names (those ending in "_") hold one comma-separated
// entry per bin.  When GLOBAL_DIR_XPRE is set, it is prefixed to every file
// name that follows it, as the reference does.
//
// A ".b16" file holds three native ints (bitj, nrows, ncols) followed by ncols
// chunks of rup(nrows, bitj)/8 bytes; chunk c holds bits 0..nrows-1 of column
// c, most significant bit first.  A_t files (nrows = SNPs, ncols = patients)
// therefore hold one patient row per chunk.
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <sys/stat.h>

#include <map>

#include "bcc_driver.h"

namespace lakbcc {

namespace {

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\n' || s[a] == '\r')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\n' || s[b - 1] == '\r')) --b;
  return s.substr(a, b - a);
}

std::vector<std::string> split_list(const std::string &v) {
  std::vector<std::string> out;
  size_t start = 0;
  for (size_t i = 0; i <= v.size(); ++i)
    if (i == v.size() || v[i] == ',') { out.push_back(trim(v.substr(start, i - start))); start = i + 1; }
  return out;
}

struct B16 {
  int bitj = 0, nrows = 0, ncols = 0;
  std::vector<unsigned char> data;  // ncols chunks of rup(nrows,bitj)/8 bytes
  long chunk() const { return bitj > 0 ? (long)(nrows + (bitj - nrows % bitj) % bitj) / 8 : 0; }
};

int read_b16(const std::string &path, B16 &b, bool header_only, std::string &err) {
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) { err = "cannot open " + path; return 2; }
  int hdr[3] = {0, 0, 0};
  if (fread(hdr, sizeof(int), 3, fp) != 3) { fclose(fp); err = "short header in " + path; return 2; }
  b.bitj = hdr[0]; b.nrows = hdr[1]; b.ncols = hdr[2];
  if (b.bitj != BITJ || b.nrows < 0 || b.ncols < 0) {
    fclose(fp);
    err = "unsupported header in " + path + " (bitj must be 16)";
    return 2;
  }
  if (!header_only) {
    const size_t n = (size_t)b.ncols * (size_t)b.chunk();
    b.data.assign(n, 0);
    if (n && fread(b.data.data(), 1, n, fp) != n) { fclose(fp); err = "short data in " + path; return 2; }
  }
  fclose(fp);
  return 0;
}

int parse_int(const std::string &v, const std::string &name, int &out, std::string &err) {
  char *end = nullptr;
  errno = 0;
  long x = strtol(v.c_str(), &end, 10);
  if (errno || end == v.c_str()) { err = "bad integer for " + name + ": '" + v + "'"; return 2; }
  out = (int)x;
  return 0;
}

int parse_double(const std::string &v, const std::string &name, double &out, std::string &err) {
  char *end = nullptr;
  errno = 0;
  double x = strtod(v.c_str(), &end);
  if (errno || end == v.c_str()) { err = "bad number for " + name + ": '" + v + "'"; return 2; }
  out = x;
  return 0;
}

// xcc_out_xdrop_load (dir_c/bcc_scorebox.c:182-200): one (row, column) pair
// per line; the number of lines is the number of newline characters.
int read_xdrop(const std::string &path, std::vector<int> &pairs, std::string &err) {
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) { err = "cannot open out_xdrop file " + path; return 2; }
  std::string text;
  char buf[65536];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, n);
  fclose(fp);
  size_t nlines = 0;
  for (char c : text) nlines += (c == '\n');
  pairs.assign(2 * nlines, 0);
  const char *p = text.c_str();
  for (size_t i = 0; i < 2 * nlines; ++i) {
    char *end = nullptr;
    const long x = strtol(p, &end, 10);
    if (end == p) { err = "bad out_xdrop line in " + path; return 2; }
    pairs[i] = (int)x;
    p = end;
  }
  return 0;
}

}  // namespace

int read_in_file(const char *path, Params &P, Input &I, std::string &err) {
  FILE *fp = fopen(path, "rb");
  if (!fp) { err = std::string("cannot open ") + path; return 2; }
  std::string text;
  char buf[65536];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, n);
  fclose(fp);

  // Statements in file order; names may repeat (last one wins, as with scanf).
  std::vector<std::pair<std::string, std::string>> st;
  size_t pos = 0;
  while (pos < text.size()) {
    const size_t eq = text.find('=', pos);
    if (eq == std::string::npos) break;
    const std::string name = trim(text.substr(pos, eq - pos));
    const size_t semi = text.find(';', eq + 1);
    const std::string value = trim(text.substr(eq + 1, (semi == std::string::npos ? text.size() : semi) - eq - 1));
    st.emplace_back(name, value);
    if (name == "END" || semi == std::string::npos) break;
    pos = semi + 1;
  }

  std::string xpre, test_type, dir_base, out_name;
  int nbins = 0, Y_n_cols = 0, T_n_cols = 1;
  std::vector<std::string> A_t, Z_t, A_rind, Z_rind, T_t, S_t, others;
  std::string A_cind, T_cind, scorebox_xdrop;
  int scramble_num = 0;
  std::vector<std::string> scramble_xdrop, scramble_rseed;
  std::vector<int> A_rows_decl, Z_rows_decl;
  int A_ncols_decl = -1;
  auto prefixed = [&](const std::string &f) { return xpre.empty() || f.empty() ? f : xpre + "/" + f; };
  auto prefixed_list = [&](const std::string &v) {
    std::vector<std::string> l = split_list(v);
    for (auto &s : l) s = prefixed(s);
    return l;
  };
  for (auto &kv : st) {
    const std::string &k = kv.first, &v = kv.second;
    int rc = 0;
    if (k == "END") break;
    else if (k == "GLOBAL_verbose" || k == "GLOBAL_thread_count" || k == "GLOBAL_omp_type" || k == "GLOBAL_LBITS") { /* host threading and logging: not used */ }
    else if (k == "GLOBAL_TEST_TYPE") test_type = v;
    else if (k == "GLOBAL_scorebox_out_xdrop") scorebox_xdrop = v;
    else if (k == "GLOBAL_scorebox_row_max") rc = parse_int(v, k, P.scorebox_row_max, err);
    else if (k == "GLOBAL_scorebox_row_num") rc = parse_int(v, k, P.scorebox_row_num, err);
    else if (k == "GLOBAL_scorebox_col_max") rc = parse_int(v, k, P.scorebox_col_max, err);
    else if (k == "GLOBAL_scorebox_col_num") rc = parse_int(v, k, P.scorebox_col_num, err);
    else if (k == "GLOBAL_scramble_num") rc = parse_int(v, k, scramble_num, err);
    else if (k == "GLOBAL_scramble_out_xdrop_") scramble_xdrop = split_list(v);
    else if (k == "GLOBAL_scramble_rseed_") scramble_rseed = split_list(v);
    else if (k == "GLOBAL_fname_bed_0in") P.bed.bed = v;
    else if (k == "GLOBAL_fname_bim_0in") P.bed.bim = v;
    else if (k == "GLOBAL_fname_fam_0in") P.bed.fam = v;
    else if (k == "GLOBAL_fname_b16_out") P.bed.b16_out = v;
    else if (k == "GLOBAL_fname_bim_out") P.bed.bim_out = v;
    else if (k == "GLOBAL_fname_fam_out") P.bed.fam_out = v;
    else if (k == "GLOBAL_n_file") rc = parse_int(v, k, P.bed.n_file, err);
    else if (k == "GLOBAL_fname_b16_0in_") P.bed.b16_in = prefixed_list(v);
    else if (k == "GLOBAL_fname_bim_0in_") P.bed.bim_in = prefixed_list(v);
    else if (k == "GLOBAL_fname_fam_0in_") P.bed.fam_in = prefixed_list(v);
    else if (k == "GLOBAL_snp_mss_threshold") rc = parse_double(v, k, P.bed.snp_mss, err);
    else if (k == "GLOBAL_snp_maf_threshold") rc = parse_double(v, k, P.bed.snp_maf, err);
    else if (k == "GLOBAL_snp_I_opt_threshold") rc = parse_double(v, k, P.bed.snp_I_opt, err);
    else if (k == "GLOBAL_pat_mss_threshold") rc = parse_double(v, k, P.bed.pat_mss, err);
    else if (k == "GLOBAL_fname_flip_flag" || k == "GLOBAL_n_fam_char_max" || k == "GLOBAL_n_bim_char_max") {
      /* the flip file is not read by the reference either; field widths are unbounded here */
    }
    else if (k == "GLOBAL_QR_strategy") P.QR_strategy = v;
    else if (k == "GLOBAL_QC_strategy") P.QC_strategy = v;
    else if (k == "GLOBAL_NBINS") rc = parse_int(v, k, nbins, err);
    else if (k == "GLOBAL_B_MLT") { rc = parse_int(v, k, P.B_MLT, err); P.D_MLT = (long long)pow(2.0, (double)P.B_MLT); }
    else if (k == "GLOBAL_D_MLT") { P.D_MLT = atoll(v.c_str()); P.B_MLT = (int)llround(log2((double)P.D_MLT)); }
    else if (k == "GLOBAL_gamma") rc = parse_double(v, k, P.gamma, err);
    else if (k == "GLOBAL_gamma_type") rc = parse_int(v, k, P.gamma_type, err);
    else if (k == "GLOBAL_kappa_squared") rc = parse_double(v, k, P.kappa_squared, err);
    else if (k == "GLOBAL_Ireq") rc = parse_int(v, k, P.Ireq, err);
    else if (k == "GLOBAL_TEST_sparse") rc = parse_int(v, k, P.test_sparse, err);
    else if (k == "GLOBAL_DIR_XPRE") xpre = v;
    else if (k == "GLOBAL_DIR_NAME") P.dir_name = v;
    else if (k == "GLOBAL_DIR_BASE") dir_base = v;
    else if (k == "GLOBAL_out_name") out_name = v;
    else if (k == "GLOBAL_A_t_name_") A_t = prefixed_list(v);
    else if (k == "GLOBAL_A_n_name_") { /* transpose of A_t: rebuilt from A_t */ }
    else if (k == "GLOBAL_Z_t_name_") Z_t = prefixed_list(v);
    else if (k == "GLOBAL_Z_n_name_") { /* transpose of Z_t: rebuilt from Z_t */ }
    else if (k == "GLOBAL_A_n_rind_") A_rind = prefixed_list(v);
    else if (k == "GLOBAL_Z_n_rind_") Z_rind = prefixed_list(v);
    else if (k == "GLOBAL_A_n_cind") A_cind = prefixed(v);
    else if (k == "GLOBAL_A_n_cols") rc = parse_int(v, k, A_ncols_decl, err);
    else if (k == "GLOBAL_A_n_rows_") { for (auto &s : split_list(v)) { int x = 0; rc |= parse_int(s, k, x, err); A_rows_decl.push_back(x); } }
    else if (k == "GLOBAL_Z_n_rows_") { for (auto &s : split_list(v)) { int x = 0; rc |= parse_int(s, k, x, err); Z_rows_decl.push_back(x); } }
    else if (k == "GLOBAL_Y_n_cols") rc = parse_int(v, k, Y_n_cols, err);
    else if (k == "GLOBAL_T_n_cols") rc = parse_int(v, k, T_n_cols, err);
    else if (k == "GLOBAL_T_t_name_") T_t = prefixed_list(v);
    else if (k == "GLOBAL_S_t_name_") S_t = prefixed_list(v);
    else if (k == "GLOBAL_T_n_name_" || k == "GLOBAL_S_n_name_") { /* transposes of T_t / S_t: rebuilt */ }
    else if (k == "GLOBAL_T_n_cind") T_cind = prefixed(v);
    else if (k == "GLOBAL_A_p_name" || k == "GLOBAL_Y_p_name" || k == "GLOBAL_Y_n_cind") {
      if (!v.empty()) others.push_back(k);
    } else if (k.rfind("GLOBAL_Y_", 0) == 0 || k.rfind("GLOBAL_W_", 0) == 0 || k.rfind("GLOBAL_T_", 0) == 0 ||
               k.rfind("GLOBAL_S_", 0) == 0) {
      for (auto &s : split_list(v)) if (!s.empty()) { others.push_back(k); break; }
    }
    if (rc) return rc;
  }
  if (test_type == "bed_to_b16" || test_type == "b16_merge") {  // lakcluster_ver18.c:361-364: no bcc inputs
    P.test_type = test_type;
    if (test_type == "b16_merge" &&
        (P.bed.n_file < 1 || (int)P.bed.b16_in.size() < P.bed.n_file || (int)P.bed.bim_in.size() < P.bed.n_file ||
         (int)P.bed.fam_in.size() < P.bed.n_file)) {
      err = "b16_merge: GLOBAL_n_file and the GLOBAL_fname_{b16,bim,fam}_0in_ lists do not agree";
      return 3;
    }
    return 0;
  }
  if (!test_type.empty() && test_type != "lakcluster_driver" && test_type != "lakcluster_scorebox" &&
      test_type != "dexcluster_driver" && test_type != "dexcluster_scorebox") {
    err = "GLOBAL_TEST_TYPE " + test_type + " is not the bcc or dexcluster driver or scorebox, bed_to_b16 or b16_merge";
    return 3;
  }
  P.test_type = test_type.empty() ? "lakcluster_driver" : test_type;
  if (!others.empty()) {
    err = "inputs not supported by this build: " + others[0] + " (extra Y/W/T/S matrices or preset allele frequencies)";
    return 4;
  }
  if (Y_n_cols > 0) { err = "Y_n_cols > 0 is not supported by this build"; return 4; }
  auto any_named = [](const std::vector<std::string> &l) {
    for (auto &x : l) if (!x.empty()) return true;
    return false;
  };
  // Covariates: every bin names its T_t and S_t files, or none does (the
  // reference's default for an absent S file with several covariate columns
  // reads past its one-row buffer).
  const bool has_T = any_named(T_t), has_S = any_named(S_t);
  if (has_T != has_S) { err = "T_t and S_t covariate files must be given together"; return 4; }
  if (P.dir_name.empty() && !out_name.empty()) {
    std::string base = dir_base;
    if (base.empty()) base = ".";
    P.dir_name = base + "/dir_" + out_name;
  }
  if (nbins <= 0 || (int)A_t.size() < nbins) { err = "GLOBAL_NBINS and GLOBAL_A_t_name_ must name one file per bin"; return 2; }
  P.nbins = nbins;
  I = Input();
  if (P.test_type == "lakcluster_scorebox" || P.test_type == "dexcluster_scorebox") {
    if (scorebox_xdrop.empty()) { err = "GLOBAL_scorebox_out_xdrop is not set"; return 2; }
    if (int rc = read_xdrop(scorebox_xdrop, I.scorebox_xdrop, err)) return rc;
  } else if (scramble_num > 0) {
    // updateglobals.c:122-135: one out_xdrop file and seed per scramble, seeds 1, 2, ... by default
    if ((int)scramble_xdrop.size() < scramble_num) { err = "GLOBAL_scramble_out_xdrop_ names fewer files than GLOBAL_scramble_num"; return 2; }
    for (int i = 0; i < scramble_num; ++i) {
      Input::Scramble sc;
      sc.rseed = (unsigned long long)(i + 1);
      if (i < (int)scramble_rseed.size() && !scramble_rseed[i].empty()) {
        int x = 0;
        if (int rc = parse_int(scramble_rseed[i], "GLOBAL_scramble_rseed_", x, err)) return rc;
        sc.rseed = (unsigned long long)(unsigned long)(long)x;
      }
      if (int rc = read_xdrop(scramble_xdrop[i], sc.xdrop, err)) return rc;
      I.scramble.push_back(std::move(sc));
    }
  }
  I.bins.resize(nbins);
  int ncols = -1;
  for (int nb = 0; nb < nbins; ++nb) {
    BinInput &B = I.bins[nb];
    B16 a;
    if (int rc = read_b16(A_t[nb], a, false, err)) return rc;
    if (ncols < 0) ncols = a.nrows;
    if (a.nrows != ncols) { err = "A_t files disagree on the number of columns"; return 2; }
    B.A_nrows = a.ncols;
    const long rb = bsize(ncols), ch = a.chunk();
    B.A_rows.assign((size_t)std::max(1, B.A_nrows) * (size_t)rb, 0);
    for (int r = 0; r < B.A_nrows; ++r) memcpy(&B.A_rows[(size_t)r * rb], &a.data[(size_t)r * ch], (size_t)ch);
    if (nb < (int)A_rind.size() && !A_rind[nb].empty()) {
      B16 m;
      if (int rc = read_b16(A_rind[nb], m, false, err)) return rc;
      if (m.nrows != B.A_nrows) { err = "row mask " + A_rind[nb] + " does not match its A_t file"; return 2; }
      B.A_mr_b.assign(bsize(B.A_nrows), 0);
      memcpy(B.A_mr_b.data(), m.data.data(), std::min(m.data.size(), B.A_mr_b.size()));
    }
    if (nb < (int)Z_t.size() && !Z_t[nb].empty()) {
      B16 z;
      if (int rc = read_b16(Z_t[nb], z, false, err)) return rc;
      if (z.nrows != ncols) { err = "Z_t file " + Z_t[nb] + " has the wrong number of columns"; return 2; }
      B.Z_nrows = z.ncols;
      B.Z_rows.assign((size_t)std::max(1, B.Z_nrows) * (size_t)rb, 0);
      for (int r = 0; r < B.Z_nrows; ++r) memcpy(&B.Z_rows[(size_t)r * rb], &z.data[(size_t)r * z.chunk()], (size_t)z.chunk());
      if (nb < (int)Z_rind.size() && !Z_rind[nb].empty()) {
        B16 m;
        if (int rc = read_b16(Z_rind[nb], m, false, err)) return rc;
        if (m.nrows != B.Z_nrows) { err = "row mask " + Z_rind[nb] + " does not match its Z_t file"; return 2; }
        B.Z_mr_b.assign(bsize(B.Z_nrows), 0);
        memcpy(B.Z_mr_b.data(), m.data.data(), std::min(m.data.size(), B.Z_mr_b.size()));
      }
    }
  }
  I.ncols = ncols;
  I.T_ncols = 1;
  if (has_T) {
    // T_t: one chunk per case row holding its T_ncols covariate bits (the
    // layout of the A_t files); S_t the same for the control rows.
    int tc = -1;
    for (int nb = 0; nb < nbins; ++nb) {
      BinInput &B = I.bins[nb];
      if (nb >= (int)T_t.size() || nb >= (int)S_t.size() || T_t[nb].empty() || S_t[nb].empty()) {
        err = "every bin needs T_t and S_t covariate files";
        return 4;
      }
      B16 t, u;
      if (int rc = read_b16(T_t[nb], t, false, err)) return rc;
      if (int rc = read_b16(S_t[nb], u, false, err)) return rc;
      if (tc < 0) tc = t.nrows;
      if (t.nrows != tc || u.nrows != tc || t.ncols != B.A_nrows || u.ncols != B.Z_nrows) {
        err = "covariate files " + T_t[nb] + " / " + S_t[nb] + " do not match their bin";
        return 2;
      }
      const long tb = bsize(tc);
      B.T_rows.assign((size_t)std::max(1, B.A_nrows) * (size_t)tb, 0);
      for (int r = 0; r < B.A_nrows; ++r) memcpy(&B.T_rows[(size_t)r * tb], &t.data[(size_t)r * t.chunk()], (size_t)t.chunk());
      B.S_rows.assign((size_t)std::max(1, B.Z_nrows) * (size_t)tb, 0);
      for (int r = 0; r < B.Z_nrows; ++r) memcpy(&B.S_rows[(size_t)r * tb], &u.data[(size_t)r * u.chunk()], (size_t)u.chunk());
    }
    I.T_ncols = tc;
    if (T_n_cols != tc) { err = "GLOBAL_T_n_cols does not match the covariate files"; return 2; }
  } else if (T_n_cols != 1) {
    err = "GLOBAL_T_n_cols > 1 needs T_t and S_t covariate files";
    return 4;
  }
  if (!T_cind.empty()) {
    // a covariate mask is accepted when it retains every column (the
    // restatement keeps every covariate column)
    B16 m;
    if (int rc = read_b16(T_cind, m, false, err)) return rc;
    if (m.nrows < I.T_ncols) { err = "covariate mask " + T_cind + " is shorter than T_ncols"; return 2; }
    for (int c = 0; c < I.T_ncols; ++c)
      if (!((m.data[c / 8] >> (7 - c % 8)) & 1)) { err = "a covariate mask that drops columns is not supported"; return 4; }
  }
  if (A_ncols_decl >= 0 && A_ncols_decl != ncols) { err = "GLOBAL_A_n_cols does not match the A_t files"; return 2; }
  if (!A_cind.empty()) {
    B16 m;
    if (int rc = read_b16(A_cind, m, false, err)) return rc;
    if (m.nrows != ncols) { err = "column mask " + A_cind + " does not match the A_t files"; return 2; }
    I.mc_b.assign(bsize(ncols), 0);
    memcpy(I.mc_b.data(), m.data.data(), std::min(m.data.size(), I.mc_b.size()));
  }
  return 0;
}

int make_output_dir(const std::string &dir) {
  if (dir.empty()) return 0;
  struct stat st;
  if (stat(dir.c_str(), &st) == -1 && mkdir(dir.c_str(), 0755) != 0) return 2;
  return 0;
}

}  // namespace lakbcc
