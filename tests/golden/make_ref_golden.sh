#!/bin/bash
# Regenerates tests/golden/ref/*.dat by running the reference programs
# themselves (built by oracle/ref_build.py into oracle/_ref/bin) on a GPU host.
#   inj_*    : injected-stream build (oracle/inj_shim.cuh): bit-exact fixtures
#   curand_* : the reference's own cuRAND build: statistical fixtures + timing
# usage (repo root, GPU host): bash tests/golden/make_ref_golden.sh [outdir]
set -euo pipefail
OUT=${1:-tests/golden/ref}
B=$PWD/oracle/_ref/bin
python oracle/ref_build.py --sizes 16,64
T=$(mktemp -d)
mkdir -p "$OUT/logs"
for p in SSC MSC; do
  $B/PAising${p}_L16_inj -R 1000 -t 10 -s 100 -o $T/a_$p > "$OUT/logs/inj_${p}_L16.log"
  cp $T/a_$p/PA_results_run_0.dat "$OUT/inj_${p}_L16_R1000_t10_d0.005_s100.dat"
  $B/PAising${p}_L16_inj -R 1000 -t 10 -s 7 -M 2 -o $T/b_$p > "$OUT/logs/inj_${p}_L16_M2.log"
  for k in 0 1; do cp $T/b_$p/PA_results_run_$k.dat "$OUT/inj_${p}_L16_R1000_t10_d0.005_s7_M2_run$k.dat"; done
  # AdaptiveStep build: dbeta is the first step, later runs replay run 0's schedule
  $B/PAising${p}_L16_inj_adaptive -R 1000 -t 10 -s 100 -o $T/e_$p > "$OUT/logs/inj_${p}_L16_adaptive.log"
  cp $T/e_$p/PA_results_run_0.dat "$OUT/inj_${p}_L16_R1000_t10_d0.005_s100_adaptive.dat"
  $B/PAising${p}_L16_inj_adaptive -R 1000 -t 10 -s 7 -M 2 -d 0.01 -o $T/f_$p > "$OUT/logs/inj_${p}_L16_M2_adaptive.log"
  for k in 0 1; do cp $T/f_$p/PA_results_run_$k.dat "$OUT/inj_${p}_L16_R1000_t10_d0.01_s7_M2_adaptive_run$k.dat"; done
  # MHR + EnergiesPopStore build: reweighted observables and per-temperature energies
  $B/PAising${p}_L16_inj_records -R 1000 -t 10 -s 100 -d 0.05 -o $T/g_$p > "$OUT/logs/inj_${p}_L16_records.log"
  mkdir -p "$OUT/inj_${p}_L16_R1000_t10_d0.05_s100_records"
  cp $T/g_$p/*.dat "$OUT/inj_${p}_L16_R1000_t10_d0.05_s100_records/"
  $B/PAising${p}_L64_inj -s 100 -o $T/c_$p > "$OUT/logs/inj_${p}_L64.log"
  cp $T/c_$p/PA_results_run_0.dat "$OUT/inj_${p}_L64_R20000_t100_d0.005_s100.dat"
  $B/PAising${p}_L64_curand -s 100 -o $T/d_$p > "$OUT/logs/cur_${p}_L64.log"
  cp $T/d_$p/PA_results_run_0.dat "$OUT/curand_${p}_L64_R20000_t100_d0.005_s100.dat"
done
# LatticePopStore build (SSC only): population text of every temperature of run 0
$B/PAisingSSC_L16_inj_lattice -R 20 -t 5 -s 100 -d 0.25 -o $T/h_SSC > "$OUT/logs/inj_SSC_L16_lattice.log"
mkdir -p "$OUT/inj_SSC_L16_R20_t5_d0.25_s100_lattice"
cp $T/h_SSC/*.dat "$OUT/inj_SSC_L16_R20_t5_d0.25_s100_lattice/"
rm -rf "$T"
