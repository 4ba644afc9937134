"""Build the reference programs PAisingSSC.cu / PAisingMSC.cu as oracle binaries.

TEST INFRASTRUCTURE ONLY.  Everything this script writes goes to oracle/_ref/
(git-ignored).  The reference sources are read where they lie; the only
changes are the ones CUDA 13 forces or the comparison needs:

* legacy texture references were removed in CUDA 12, so the Boltzmann /
  threshold table bound to ``boltzT`` (PAisingSSC.cu:59,90-94,175,187,477,797;
  PAisingMSC.cu:63,222-223,255-256,636) becomes a ``__device__`` pointer that
  is set with cudaMemcpyToSymbol instead of cudaBindTexture;
* ``#define L 64`` (PAisingSSC.cu:27, PAisingMSC.cu:26) is compile-time in the
  reference, so one binary is built per lattice size;
* the ``inj`` variants are compiled with ``-include inj_shim.cuh``, which swaps
  cuRAND's Philox state for the injected stream H (see inj_stream.h).  The
  ``curand`` variants keep cuRAND and are the reference's own GPU build;
* the ``inj_adaptive`` variants (L=16) also define ``AdaptiveStep``, the
  reference's compile-time switch for its adaptive temperature step
  (PAisingSSC.cu:23, PAisingMSC.cu:23); the ``inj_records`` variants define
  ``MHR`` and ``EnergiesPopStore`` (multi-histogram reweighting and the
  per-temperature energy files, PAisingSSC.cu:22,24); the ``inj_lattice``
  variant (SSC, L=16) defines ``LatticePopStore`` (PAisingSSC.cu:25).

Step 1 (patch) needs the reference checkout and runs in the build container;
step 2 (nvcc) runs wherever the patched sources are, e.g. on the GPU host,
which does not have the reference checkout.

usage: python oracle/ref_build.py [--reference DIR] [--patch-only] [--sizes 16,64] [--jobs N]

DIR is the reference checkout (the directory holding PAisingSSC.cu and
PAisingMSC.cu), from --reference or the environment variable
PAISING_REFERENCE_DIR; without one, the patched copies already under
oracle/_ref/src are compiled.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ENV = "PAISING_REFERENCE_DIR"
OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(OUT, "src")
BIN_OUT = os.path.join(OUT, "bin")
DEFAULT_SIZES = (16, 64)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# (pattern, replacement, expected count) per program
_COMMON = [
    (r"CUDAErrChk\( cudaUnbindTexture\(boltzT\) \);", "CUDAErrChk( cudaSuccess );", 1),
]
_SSC = [
    (r"texture<int2,1,cudaReadModeElementType> boltzT;", "__device__ const double* boltzT;", 1),
    (r"fetch_double\(texture<int2,1> t, int i\)", "fetch_double(const double* t, int i)", 1),
    (r"int2 v = tex1Dfetch\(t,i\);", "return t[i];", 1),
    (r"return __hiloint2double\(v\.y, v\.x\);", "", 1),
    (r"CUDAErrChk\( cudaBindTexture\(NULL,boltzT,boltztext,boltzTableL \* sizeof\(double\)\) \);",
     "CUDAErrChk( cudaMemcpyToSymbol(boltzT,&boltztext,sizeof(boltztext)) );", 1),
]
_MSC = [
    (r"texture<unsigned int,1,cudaReadModeElementType> boltzT;",
     "__device__ const unsigned int* boltzT;", 1),
    (r"tex1Dfetch\(boltzT, ([01])\)", r"boltzT[\1]", 4),
    (r"CUDAErrChk\( cudaBindTexture\(NULL,boltzT,boltztext,boltzTableL \* sizeof\(unsigned int\)\) \);",
     "CUDAErrChk( cudaMemcpyToSymbol(boltzT,&boltztext,sizeof(boltztext)) );", 1),
]


def _patch(text: str, rules, L: int) -> str:
    for pat, rep, n in rules + _COMMON:
        text, k = re.subn(pat, rep, text)
        if k != n:
            raise RuntimeError(f"pattern {pat!r}: {k} matches, expected {n}")
    text, k = re.subn(r"^#define L\s+64\b", f"#define L\t{L}", text, flags=re.M)
    if k != 1:
        raise RuntimeError("#define L not found")
    return text


def reference_dir(explicit: str | None = None) -> str | None:
    """The reference checkout: the given directory, else $PAISING_REFERENCE_DIR;
    None when neither names a directory holding both programs."""
    d = explicit or os.environ.get(REF_ENV)
    if d and all(os.path.isfile(os.path.join(d, f"PAising{p}.cu")) for p in ("SSC", "MSC")):
        return d
    return None


def patch(sizes, ref_dir: str) -> None:
    os.makedirs(SRC_OUT, exist_ok=True)
    for prog, rules in (("SSC", _SSC), ("MSC", _MSC)):
        with open(os.path.join(ref_dir, f"PAising{prog}.cu")) as f:
            text = f.read()
        for L in sizes:
            with open(os.path.join(SRC_OUT, f"PAising{prog}_L{L}.cu"), "w") as f:
                f.write(_patch(text, rules, L))
    shutil.copy(os.path.join(HERE, "inj_shim.cuh"), SRC_OUT)
    shutil.copy(os.path.join(HERE, "inj_stream.h"), SRC_OUT)


def _compile(src: str, variant: str) -> str:
    base = os.path.splitext(os.path.basename(src))[0]
    out = os.path.join(BIN_OUT, f"{base}_{variant}")
    cmd = ["nvcc", "-O3", ARCH, "-w", "-o", out, src]
    if variant.startswith("inj"):
        cmd[1:1] = ["-include", os.path.join(SRC_OUT, "inj_shim.cuh"), "-I", SRC_OUT]
    if variant.endswith("adaptive"):  # the reference's AdaptiveStep build (its line 23 switch)
        cmd[1:1] = ["-DAdaptiveStep"]
    if variant.endswith("records"):  # its MHR and EnergiesPopStore builds (lines 22, 24)
        cmd[1:1] = ["-DMHR", "-DEnergiesPopStore"]
    if variant.endswith("lattice"):  # its LatticePopStore build (PAisingSSC.cu line 25; SSC only)
        cmd[1:1] = ["-DLatticePopStore"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {out}:\n{r.stderr[-2000:]}")
    return out


def compile_all(jobs: int, sizes) -> list[str]:
    """Compiles the patched sources of the given lattice sizes (every variant
    that exists for them)."""
    os.makedirs(BIN_OUT, exist_ok=True)
    want = tuple(f"_L{L}.cu" for L in sizes)
    srcs = sorted(f for f in os.listdir(SRC_OUT) if f.startswith("PAising") and f.endswith(want))
    tasks = [(os.path.join(SRC_OUT, s), v) for s in srcs for v in ("inj", "curand")]
    tasks += [(os.path.join(SRC_OUT, s), v) for s in srcs if s.endswith("_L16.cu") for v in ("inj_adaptive", "inj_records")]
    tasks += [(os.path.join(SRC_OUT, s), "inj_lattice") for s in srcs if s == "PAisingSSC_L16.cu"]
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        return list(ex.map(lambda a: _compile(*a), tasks))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help=f"reference checkout (default: ${REF_ENV})")
    ap.add_argument("--patch-only", action="store_true")
    ap.add_argument("--sizes", default=",".join(map(str, DEFAULT_SIZES)))
    ap.add_argument("--jobs", type=int, default=min(8, os.cpu_count() or 1))
    a = ap.parse_args(argv)
    sizes = [int(s) for s in a.sizes.split(",") if s]
    ref = reference_dir(a.reference)
    if ref:
        patch(sizes, ref)
    elif not os.path.isdir(SRC_OUT):
        print("reference sources unavailable and no patched copy present", file=sys.stderr)
        return 1
    if not a.patch_only:
        for b in compile_all(a.jobs, sizes):
            print(b)
    return 0


if __name__ == "__main__":
    sys.exit(main())
