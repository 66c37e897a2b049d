#!/usr/bin/env bash
# build_ref.sh — compiles the reference program for the host CPU (test oracle
# pin; TEST INFRASTRUCTURE ONLY).
#
# Reads the reference sources where they lie (the directory named by the
# REF_SRC environment variable; there is no default) and writes only into
# oracle/_ref/ (git-ignored):
#   oracle/_ref/gen/ref_fixA.cpp   cuda_Cell_Detailed.cu with
#       - the "fixA" repair: lines 1475-1597 (the second, duplicated dyad /
#         cytosol block) and the stray brace on line 1692 deleted, which is the
#         minimum that makes the file compile;
#       - the lattice / protocol macros nx, ny, nz, nbeat, tperid guarded by
#         #ifndef so that each build variant can set them with -D;
#       - the <<<grid,block>>> launches turned into REF_LAUNCH(...) calls of the
#         host shim (oracle/ref_shim/ref_shim.h), Compute counted as one step;
#       - the linescan plane (hard-coded jz = 5) and the RNG seed (18) made
#         overridable, and the time loop bounded by REF_MAX_STEPS when set;
#       - the NCX call of Compute (:1296) routed through REF_NCX, so that a
#         variant can select the reference's oldncx or ncx_noallo instead.
#   oracle/_ref/gen/*.c, reesica.h   the three device files it includes, copied
#       so that the generated program builds where the reference is absent
#       (REF_SRC unset: the generated copy is used when it exists).
#   oracle/_ref/ref_<variant>         host executables (g++ -fopenmp).
# The LCC loop of Compute tests lcc[ll] < 16 before ll < 8 (:1253), so a CRU
# with all eight slots filled (iso after 5.5 PCL, randomlcc) reads lcc[8], one
# int past the array.  g++ -O2 takes that read as proof that ll < 8 always
# holds, drops the bound and runs the loop on through nl, nou, ncu ...;
# -fno-aggressive-loop-optimizations keeps the bound, so the loop stops after
# slot 8 as written.
# Usage: build_ref.sh [variant ...]   (default: all variants below)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_SRC="${REF_SRC:-}"
OUT="$HERE/_ref"
GEN="$OUT/gen"
CXX="${CXX:-g++}"
mkdir -p "$GEN"

if [ -n "$REF_SRC" ] && [ -f "$REF_SRC/cuda_Cell_Detailed.cu" ]; then
  sed -e '1475,1597d' -e '1692d' "$REF_SRC/cuda_Cell_Detailed.cu" |
    sed -E \
      -e 's/^#define (nbeat|tperid|nx|ny|nz)([[:space:]]+)([^/]*)(.*)$/#ifndef \1\n#define \1 \3 \4\n#endif/' \
      -e 's/Init<<<numBlocks, threadsPerBlock>>>\((.*)\);/REF_LAUNCH(Init(\1));/' \
      -e 's/setup_kernel<<<numBlocks,threadsPerBlock>>>\(18,(.*)\);/REF_LAUNCH(setup_kernel(REF_SEED,\1));/' \
      -e 's/Compute<<<numBlocks, threadsPerBlock>>>\((.*)\);/REF_LAUNCH_STEP(Compute(\1));/' \
      -e 's/int jz = 5;/int jz = REF_LINESCAN_JZ;/' \
      -e 's/while \(t<nbeat\*tperid\+2100\)\{/while (t<nbeat*tperid+2100 \&\& ref_continue()){/' \
      -e 's/CRU\[ac\]\.xinaca=sv_ncx\*svncx_lqt\*ncx\(/CRU[ac].xinaca=sv_ncx*svncx_lqt*REF_NCX(/' \
      > "$GEN/ref_fixA.cpp.tmp"
  for f in subroutine_cuda.c reesica.h buffers.c; do cp "$REF_SRC/$f" "$GEN/$f"; done
  mv "$GEN/ref_fixA.cpp.tmp" "$GEN/ref_fixA.cpp"
elif [ ! -f "$GEN/ref_fixA.cpp" ]; then
  echo "build_ref.sh: no reference sources (REF_SRC='$REF_SRC') and no generated copy in $GEN" >&2
  exit 3
fi

for pat in 'REF_LAUNCH_STEP(Compute' 'REF_LAUNCH(Init' 'REF_LAUNCH(setup_kernel' 'REF_LINESCAN_JZ' 'ref_continue' 'svncx_lqt\*REF_NCX('; do
  grep -q "$pat" "$GEN/ref_fixA.cpp" || { echo "build_ref.sh: patch '$pat' did not apply" >&2; exit 4; }
done

# variant name -> compile definitions
declare -A VARIANTS=(
  # 20x10x5 control build, PCL 400 ms, 2 beats (the CPU-sized lattice)
  [c1]="-Dnx=20 -Dny=10 -Dnz=5 -Dnbeat=2 -Dtperid=400.0 -DREF_LINESCAN_JZ=2"
  # same lattice, the run.sh build (make il: -Diso2 -Dlqt)
  [c1_il]="-Dnx=20 -Dny=10 -Dnz=5 -Dnbeat=2 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -Diso2 -Dlqt"
  # 12x9x7 lattice, make il, PCL 1000 ms, 1 beat (small and fast)
  [small_il]="-Dnx=12 -Dny=9 -Dnz=7 -Dnbeat=1 -Dtperid=1000.0 -DREF_LINESCAN_JZ=5 -Diso2 -Dlqt"
  # the shipped 64x28x12 make-il build
  [default_il]="-Diso2 -Dlqt -DREF_LINESCAN_JZ=5"
  # the mean lattice of the 512-cell heterogeneous ensemble (80x16x8, 6552
  # interior CRUs), iso2 build, PCL 1750 ms: the CPU baseline of bench.py
  [bench_mean]="-Dnx=80 -Dny=16 -Dnz=8 -Dnbeat=20 -Dtperid=1750.0 -DREF_LINESCAN_JZ=5 -Diso2"
  # small_il with the reference's cadist_ writer enabled (#define outputcadist)
  [small_il_cd]="-Dnx=12 -Dny=9 -Dnz=7 -Dnbeat=1 -Dtperid=1000.0 -DREF_LINESCAN_JZ=5 -Diso2 -Dlqt -Doutputcadist"
  # the voltage protocols and cell preparations of the reference's build
  # switches (:34-35, :54-61), each on a small lattice
  [vclamp]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -Dvclamp"
  [brownvclamp]="-Dnx=6 -Dny=5 -Dnz=4 -Dnbeat=2 -Dtperid=3000.0 -DREF_LINESCAN_JZ=2 -Dbrownvclamp"
  [apclamp]="-Dnx=10 -Dny=6 -Dnz=5 -Dnbeat=2 -Dtperid=200.0 -DREF_LINESCAN_JZ=2 -Diso2 -Dlqt -Dapclamp"
  [linearapclamp]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=1000.0 -DREF_LINESCAN_JZ=2 -Dlinearapclamp"
  [nopacing]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -Diso2 -Dlqt -Dnopacing"
  [perm]="-Dnx=12 -Dny=9 -Dnz=6 -Dnbeat=1 -Dtperid=1000.0 -DREF_LINESCAN_JZ=3 -Dperm"
  # the rarer builds: time-dependent isoproterenol (alone and with make il),
  # slowncxchange, and the two NCX functions no build calls
  [iso]="-Dnx=8 -Dny=6 -Dnz=5 -Dnbeat=13 -Dtperid=100.0 -DREF_LINESCAN_JZ=2 -Diso"
  [iso_il]="-Dnx=8 -Dny=6 -Dnz=5 -Dnbeat=13 -Dtperid=100.0 -DREF_LINESCAN_JZ=2 -Diso -Diso2 -Dlqt"
  [slowncxchange]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -Dslowncxchange"
  [oldncx]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -DREF_NCX_OLD"
  [ncx_noallo]="-Dnx=12 -Dny=8 -Dnz=5 -Dnbeat=1 -Dtperid=400.0 -DREF_LINESCAN_JZ=2 -DREF_NCX_NOALLO"
)
want=("$@")
if [ ${#want[@]} -eq 0 ]; then want=("${!VARIANTS[@]}"); fi
pids=()
for v in "${want[@]}"; do
  defs="${VARIANTS[$v]:?unknown variant $v}"
  # shellcheck disable=SC2086
  $CXX -std=c++17 -O2 -fno-aggressive-loop-optimizations -fopenmp -ffp-contract=off -w -x c++ \
    -include "$HERE/ref_shim/ref_shim.h" -I "$HERE/ref_shim/include" -I "$GEN" \
    -DREF_SEED=18 $defs "$GEN/ref_fixA.cpp" -o "$OUT/ref_$v" -lm &
  pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
