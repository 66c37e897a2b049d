// cli_main.cpp — drop-in replacement for the reference program
// cuda_Cell_Detailed (cuda_Cell_Detailed.cu:232-1105).
//
//   cuda_Cell_Detailed <device> <name> a3 a4 a5 a6 a7 a8 a9 a10 [options]
//
// Positional arguments keep the reference's meaning (run.sh:7-9):
//   a3 clamp voltage, a4 cjsr_basal, a5 NCX scale, a6 Ku, a7 r1 (unused),
//   a8 Kb, a9 ICaL scale, a10 Ku2.
// Writes wholetest_<name>, linescan_<name> and cadist_<name> in the same
// formats (cadist_ stays empty, as in the reference's default build, unless
// --cadist selects the outputcadist build), prints "Initialization Complete"
// and exits 0.  The reference's compile-time switches become
// options; the defaults are the run.sh build (make il) on the shipped
// 64x28x12 lattice, PCL 4000 ms, 7 beats:
//   --nx N --ny N --nz N --nbeats N --pcl MS   lattice and protocol
//   --lqt 0|1 --iso2 0|1 --tapsi 0|1           build modes (Makefile:8-28)
//   --cadist                                   outputcadist build (:1001-1013)
//   --no-linescan                              build without outputlinescan (:46):
//                                              linescan_<name> stays empty
//   --protocol paced|nopacing|vclamp|brownvclamp|apclamp|linearapclamp
//                                              voltage protocol build (:34, :54-61);
//                                              vclamp holds a3 mV after 100 ms,
//                                              apclamp reads v_1000.txt (:383-395)
//   --perm                                     permeabilised-cell build (:35)
//   --iso --randomlcc --slowncxchange          the -Diso, -Drandomlcc and
//                                              -Dslowncxchange builds (:31-32, :52)
//   --ncx ncx|oldncx|ncx_noallo                NCX function (subroutine_cuda.c:47-120)
//   --mixed                                    FP32 lattice / FP64 whole-cell
//   --seed S --ikr-scale X --cao MM --linescan-jz J --max-steps N
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "rh.h"

static void usage() {
  fprintf(stderr,
          "usage: cuda_Cell_Detailed <device> <name> a3 a4 a5 a6 a7 a8 a9 a10 [--nx N] [--ny N] "
          "[--nz N] [--nbeats N] [--pcl MS] [--lqt 0|1] [--iso2 0|1] [--tapsi 0|1] [--cadist] [--no-linescan] [--protocol P] [--perm] [--iso] [--randomlcc] "
          "[--slowncxchange] [--ncx F] [--mixed] "
          "[--seed S] [--ikr-scale X] [--cao MM] [--linescan-jz J] [--max-steps N]\n");
}

int main(int argc, char** argv) {
  if (argc < 11) {
    usage();
    return 2;
  }
  rh_cell_params p;
  rh_default_cell_params(&p);
  rh_run_opts o;
  rh_default_run_opts(&o);
  int dev = atoi(argv[1]);
  o.device = dev >= 0 ? dev : 0;  // :236-242
  std::string name = argv[2];
  p.clamp_mv = atof(argv[3]);
  p.cjsr_basal = atof(argv[4]);
  p.ncx_scale = atof(argv[5]);
  p.ku = atof(argv[6]);
  p.r1 = atof(argv[7]);
  p.kb = atof(argv[8]);
  p.ica_scale = atof(argv[9]);
  p.ku2 = atof(argv[10]);
  long long max_steps = -1;
  for (int a = 11; a < argc; ++a) {
    std::string k = argv[a];
    auto next = [&]() -> const char* {
      if (a + 1 >= argc) {
        usage();
        exit(2);
      }
      return argv[++a];
    };
    if (k == "--nx") p.nx = atoi(next());
    else if (k == "--ny") p.ny = atoi(next());
    else if (k == "--nz") p.nz = atoi(next());
    else if (k == "--nbeats") p.nbeats = atoi(next());
    else if (k == "--pcl") p.pcl_ms = atof(next());
    else if (k == "--lqt") p.lqt = atoi(next());
    else if (k == "--iso2") p.iso2 = atoi(next());
    else if (k == "--tapsi") p.tapsi = atoi(next());
    else if (k == "--mixed") o.precision = RH_MIXED;
    else if (k == "--cadist") o.record_cadist = 1;
    else if (k == "--no-linescan") o.record_linescan = 0;
    else if (k == "--perm") p.perm = 1;
    else if (k == "--iso") p.iso = 1;
    else if (k == "--randomlcc") p.randomlcc = 1;
    else if (k == "--slowncxchange") p.slowncx = 1;
    else if (k == "--ncx") {
      const std::string v = next();
      if (v == "ncx") p.ncx_form = RH_NCX_ALLOSTERIC;
      else if (v == "oldncx") p.ncx_form = RH_NCX_OLD;
      else if (v == "ncx_noallo") p.ncx_form = RH_NCX_NOALLO;
      else {
        usage();
        return 2;
      }
    }
    else if (k == "--protocol") {
      const std::string v = next();
      if (v == "paced") p.protocol = RH_PROTO_PACED;
      else if (v == "nopacing") p.protocol = RH_PROTO_NOPACING;
      else if (v == "vclamp") p.protocol = RH_PROTO_VCLAMP;
      else if (v == "brownvclamp") p.protocol = RH_PROTO_BROWN_VCLAMP;
      else if (v == "apclamp") p.protocol = RH_PROTO_AP_CLAMP;
      else if (v == "linearapclamp") p.protocol = RH_PROTO_LINEAR_AP_CLAMP;
      else {
        usage();
        return 2;
      }
    }
    else if (k == "--seed") p.seed = (uint32_t)strtoul(next(), nullptr, 10);
    else if (k == "--ikr-scale") p.ikr_scale = atof(next());
    else if (k == "--cao") p.cao_mM = atof(next());
    else if (k == "--linescan-jz") p.linescan_jz = atoi(next());
    else if (k == "--max-steps") max_steps = atoll(next());
    else {
      usage();
      return 2;
    }
  }
  FILE* fw = fopen(("wholetest_" + name).c_str(), "w");
  FILE* fl = fopen(("linescan_" + name).c_str(), "w");
  FILE* fc = fopen(("cadist_" + name).c_str(), "w");
  if (!fw || !fl || !fc) {
    fprintf(stderr, "cannot open output files for %s\n", name.c_str());
    return 1;
  }
  o.window_steps = 100;
  o.output_capacity = 64;
  o.cadist_capacity = 8;  // one record per 200 steps at most; drained every 100
  rh_sim* sim = nullptr;
  int rc = rh_create(&p, 1, &o, &sim);
  if (rc != RH_OK) {
    char buf[512];
    rh_last_error(nullptr, buf, sizeof buf);
    fprintf(stderr, "rh_create failed: %s\n", buf);
    return 1;
  }
  if (p.protocol == RH_PROTO_AP_CLAMP) {  // :383-395: one PCL of samples from v_1000.txt
    const int numsteps = (int)(p.pcl_ms / o.dt_ms + 0.1);
    std::vector<double> varray(numsteps);
    FILE* fv = fopen("v_1000.txt", "r");
    int got = 0;
    if (fv) {
      while (got < numsteps && fscanf(fv, "%lf", &varray[got]) == 1) ++got;
      fclose(fv);
    }
    if (got < numsteps) {
      fprintf(stderr, "v_1000.txt: %d of the %d voltages the AP clamp needs\n", got, numsteps);
      rh_destroy(sim);
      return 1;
    }
    if (rh_set_ap_clamp(sim, 0, varray.data(), numsteps) != RH_OK) {
      char buf[512];
      rh_last_error(sim, buf, sizeof buf);
      fprintf(stderr, "%s\n", buf);
      rh_destroy(sim);
      return 1;
    }
  }
  printf("Initialization Complete\n");
  fflush(stdout);
  const int lx = p.nx - 2;
  std::vector<double> wc(64 * RH_WHOLECELL_COLS), ls((size_t)64 * lx * RH_LINESCAN_COLS);
  const size_t ncru = (size_t)(p.nx - 2) * (p.ny - 2) * (p.nz - 2);
  const size_t cd_len = 2 + RH_CADIST_COLS * ncru;
  std::vector<double> cd(o.record_cadist ? 8 * cd_len : 0);
  char line[4096];
  long long steps = 0;
  uint32_t reported = 0;
  for (;;) {
    long long chunk = 100;
    if (max_steps >= 0) chunk = std::min(chunk, max_steps - steps);
    if (chunk <= 0) break;
    rc = rh_run_steps(sim, chunk);
    if (rc != RH_OK) break;
    steps += chunk;
    int32_t nrec = 0, nls = 0;
    rc = rh_drain_wholecell(sim, 0, wc.data(), 64, &nrec);
    if (rc != RH_OK) break;
    rc = rh_drain_linescan(sim, 0, ls.data(), 64, &nls);
    if (rc != RH_OK) break;
    if (o.record_cadist) {  // :1005, :1009
      int32_t ncd = 0;
      rc = rh_drain_cadist(sim, 0, cd.data(), 8, &ncd);
      if (rc != RH_OK) break;
      for (int r = 0; r < ncd; ++r) {
        const double* rec = &cd[(size_t)r * cd_len];
        fprintf(fc, "0 header %f %f\n", rec[0], rec[1]);
        for (size_t k = 0; k < ncru; ++k) {
          const double* v = rec + 2 + RH_CADIST_COLS * k;
          fprintf(fc, "%f %f %f %f %f %f\n", v[0], v[1], v[2], v[3], v[4], v[5]);
        }
      }
      fflush(fc);
    }
    for (int r = 0; r < nrec; ++r) {
      if (r < nls) {
        for (int x = 0; x < lx; ++x) {
          rh_format_linescan(&ls[((size_t)r * lx + x) * RH_LINESCAN_COLS], line, sizeof line);
          fputs(line, fl);
        }
        fputs("\n", fl);
        fflush(fl);
      }
      rh_format_wholecell(&wc[(size_t)r * RH_WHOLECELL_COLS], line, sizeof line);
      fputs(line, fw);
      fflush(fw);
    }
    uint32_t st = 0;
    rc = rh_cell_status(sim, 0, &st);
    if (rc != RH_OK) break;
    if ((st & RH_STATUS_CI_HIGH) && !(reported & RH_STATUS_CI_HIGH)) {
      rh_membrane m;
      rh_get_membrane(sim, 0, &m);
      printf("%g error!\n", m.t);  // the reference's ci > 1000 diagnostic (:878-880)
      reported |= RH_STATUS_CI_HIGH;
    }
    if (st & RH_STATUS_DONE) break;
  }
  if (rc != RH_OK) {
    char buf[512];
    rh_last_error(sim, buf, sizeof buf);
    fprintf(stderr, "simulation failed: %s\n", buf);
  }
  fclose(fw);
  fclose(fl);
  fclose(fc);
  rh_destroy(sim);
  return rc == RH_OK ? 0 : 1;
}
