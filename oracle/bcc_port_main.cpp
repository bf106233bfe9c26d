// Test infrastructure: the package's bcc solve driver linked against the
// plain-C oracle kernels (lak_oracle.c via lak_oracle_wrap.c).  Builds on
// x86-64 and aarch64; used for the CPU baseline of whole solves and as a
// reference-independent check of the GPU library's solve outputs.
//
// usage: lakbcc_port file.in [threads]
#include <stdio.h>
#include <stdlib.h>

#include "../lakcluster_c_gb300/csrc/bcc_driver.h"
#include "lak_oracle.h"

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s file.in [threads]\n", argv[0]);
    return 2;
  }
  lakbcc::Params P;
  lakbcc::Input I;
  lakbcc::Output O;
  std::string err;
  int rc = lakbcc::read_in_file(argv[1], P, I, err);
  if (rc) { fprintf(stderr, "error: %s\n", err.c_str()); return rc; }
  if (argc > 2) lako_set_threads(atoi(argv[2]));
  lako_set_d_mlt(P.D_MLT);
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
