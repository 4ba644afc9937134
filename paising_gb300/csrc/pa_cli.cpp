// pa_cli.cpp -- command-line driver with the reference programs' interface.
//
// Same options, defaults, output directory and results files as PAisingSSC /
// PAisingMSC (PAisingSSC.cu:367-404, 406-416, 670-692, 801-806), on top of the
// C ABI in include/paising.h.  L is a compile-time #define in the reference
// (PAisingSSC.cu:27); here it is the extra option -L.  Further extensions:
// -c ssc|msc (coding), -m native|reference (random stream), -w fp32|fp64
// (resampling weights), -g 0|1 (host-stepped or graph), -D device, -a (the
// adaptive temperature step of the reference's AdaptiveStep build, with its
// output directory ./data%s_L%d_R%d_EqSw%d/, PAisingSSC.cu:406-410), -T (time
// the tile sizes and SSC spins per word before the run, pa_autotune), -H (multi-histogram
// reweighting, the MHR build: PA_MHR_results_run_<r>.dat), -E (energies of
// every temperature, the EnergiesPopStore build: PA_energies_<i>.dat), -F
// (family statistics, PA_family_run_<r>.dat; not in the reference), -S (the
// LatticePopStore build: PA_lattice_<i>.dat of run 0).
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>

#include "paising.h"

static void usage(const char* prog) {
  std::printf(
      " Usage: %s [options]\n"
      " Note: all of the options are optional.\n"
      " Possible command line options are:\n\n"
      " -R Rinit           ( Rinit           = initial size of population of replicas )\n"
      " -t EQsweeps        ( EQsweeps        = number of equilibration sweeps )\n"
      " -d dBinit          ( dBinit          = inverse temperature step )\n"
      " -f Bfin            ( Bfin            = final value of inverse temperature )\n"
      " -M runs            ( runs            = number of population annealing algorithm independent runs )\n"
      " -s RNGseed         ( RNGseed         = seed for random number generation )\n"
      " -P OutputPrecision ( OutputPrecision = precision (number of digits) of the output )\n"
      " -o dataDirectory   ( dataDirectory   = data directory name )\n"
      " -L L               ( L               = linear lattice size, default 64 )\n"
      " -c ssc|msc         ( spin coding, default msc )\n"
      " -m native|reference( random stream, default native )\n"
      " -w fp32|fp64       ( resampling weights, default fp32 )\n"
      " -g 0|1             ( 1: one CUDA graph per run (default), 0: host steps each temperature )\n"
      " -D device          ( CUDA device ordinal )\n"
      " -a                 ( adaptive temperature step, MinOverlap 0.85, MaxOverlap 0.87 )\n"
      " -T                 ( autotune the sweep's tile sizes and SSC spins per word before the run )\n"
      " -H                 ( multi-histogram reweighting: PA_MHR_results_run_<r>.dat )\n"
      " -E                 ( store the energies of every temperature: PA_energies_<i>.dat )\n"
      " -F                 ( family statistics of every temperature: PA_family_run_<r>.dat )\n"
      " -S                 ( store the lattices of every temperature of run 0: PA_lattice_<i>.dat )\n",
      prog);
}

int main(int argc, char** argv) {
  pa_config c;
  pa_config_init(&c);
  c.coding = PA_CODING_MSC;
  c.seed = (uint64_t)time(nullptr);  // RNGseed = time(NULL) (PAisingSSC.cu:31)
  int precision = 11;
  bool tune = false, lattices = false;
  std::string dir;
  int opt;
  opterr = 0;
  while ((opt = getopt(argc, argv, "R:t:d:f:M:s:P:o:L:c:m:w:g:D:aTHEFS?")) != -1) {
    int i;
    double f;
    switch (opt) {  // same acceptance rules as PAisingSSC.cu:390-398
      case 'R': if ((i = std::atoi(optarg))) c.R = i; break;
      case 't': c.sweeps = std::atoi(optarg); break;
      case 'd': if ((f = std::atof(optarg)) > 0.0) c.dbeta = f; break;
      case 'f': if ((f = std::atof(optarg)) > 0.0) c.beta_final = f; break;
      case 'M': if ((i = std::atoi(optarg))) c.runs = i; break;
      case 's': if ((i = std::atoi(optarg))) c.seed = (uint64_t)(long long)i; break;
      case 'P': if ((i = std::atoi(optarg))) precision = i; break;
      case 'o': dir = optarg; if (dir.empty() || dir.back() != '/') dir += '/'; break;
      case 'L': c.L = std::atoi(optarg); break;
      case 'c': c.coding = std::strcmp(optarg, "ssc") == 0 ? PA_CODING_SSC : PA_CODING_MSC; break;
      case 'm': c.rng_mode = std::strcmp(optarg, "reference") == 0 ? PA_RNG_REFERENCE : PA_RNG_NATIVE; break;
      case 'w': c.weights = std::strcmp(optarg, "fp64") == 0 ? PA_WEIGHTS_FP64 : PA_WEIGHTS_FP32; break;
      case 'g': c.graph = std::atoi(optarg) != 0; break;
      case 'D': c.device = std::atoi(optarg); break;
      case 'a': c.adaptive = 1; break;
      case 'T': tune = true; break;
      case 'H': c.mhr = 1; break;
      case 'E': c.store_energies = 1; break;
      case 'F': c.family = 1; break;
      case 'S': lattices = true; break;
      default:
        if (optopt && optopt != '?') std::printf("illegal option -- %c\n", optopt);
        usage(argv[0]);
        return 1;
    }
  }
  if (optind < argc) {
    for (int k = optind; k < argc; ++k) std::fprintf(stderr, "Non-option argument %s\n", argv[k]);
    return 1;
  }
  const char* tag = c.coding == PA_CODING_MSC ? "MSC" : "SSC";
  if (dir.empty()) {  // ./dataSSC_L%d_R%d_EqSw%d[_dB%f]/ (PAisingSSC.cu:406-410)
    char buf[256];
    if (c.adaptive) std::snprintf(buf, sizeof(buf), "./data%s_L%d_R%d_EqSw%d/", tag, c.L, c.R, c.sweeps);
    else std::snprintf(buf, sizeof(buf), "./data%s_L%d_R%d_EqSw%d_dB%f/", tag, c.L, c.R, c.sweeps, c.dbeta);
    dir = buf;
  }
  mkdir(dir.c_str(), 0777);
  std::printf("RNG initial seed: %llu\n", (unsigned long long)c.seed);
  const double N = (double)c.L * c.L;
  const double per = c.coding == PA_CODING_MSC ? N / 8.0 : N;  // bytes of spins per replica
  std::printf("Memory use of one replica: %g kB \n", per / 1024.0);
  std::printf("Memory use of the entire population of %d replicas: %g MB \n", c.R, c.R * per / 1024.0 / 1024.0);
  std::fflush(stdout);

  pa_handle* h = nullptr;
  int st = pa_create(&c, &h);
  if (st) {
    std::fprintf(stderr, "Error: %s (%s)\n", pa_status_string(st), pa_last_error(nullptr));
    return 1;
  }
  if (tune) st = pa_autotune(h, nullptr, 0);
  if (!st && lattices) st = pa_set_lattice_dump(h, dir.c_str(), precision);
  if (!st) st = pa_run(h);
  if (st) {
    std::fprintf(stderr, "Error: %s (%s)\n", pa_status_string(st), pa_last_error(h));
    pa_destroy(h);
    return 1;
  }
  st = pa_write_results(h, dir.c_str(), precision);
  double ms = 0, att = 0;
  pa_get_timing(h, &ms, &att);
  pa_destroy(h);
  if (st) {
    std::fprintf(stderr, "Error: cannot write results to %s\n", dir.c_str());
    return 1;
  }
  std::printf("Elapsed time: %.8g s\n", ms / 1000.0);
  std::printf("Time per spin-flip: %.8g ns\n", ms * 1e6 / att);
  return 0;
}
