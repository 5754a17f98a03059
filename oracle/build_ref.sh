#!/usr/bin/env bash
# build_ref.sh -- TEST INFRASTRUCTURE ONLY.
#
# Compiles the reference's own CPU beamformer (cpu.cxx, arraysizes.cxx,
# adler32.c) from the reference sources, unmodified, once per problem shape.
# The reference fixes its shape as constexpr globals (arraysizes.hxx:22-27), so
# each shape gets a generated copy of that header under oracle/_ref/<shape>/
# with only those five numbers changed; it is force-included ahead of the
# sources, whose own include guard then skips the stock header.
# Flags follow the reference Makefile (Makefile:10-11).  Outputs go only to
# oracle/_ref/ (git-ignored).
#
# usage: oracle/build_ref.sh [REFERENCE_DIR]
#   REFERENCE_DIR defaults to $BF_REFERENCE_DIR, else the checkout this
#   recipe was written against (/root/reference).
#   builds   oracle/_ref/<T>_<F>_<D>_<P>_<B>/cpu     (stock program, prints checksum)
#            oracle/_ref/<T>_<F>_<D>_<P>_<B>/ref_io  (reads E/A/G files, writes J)
#   and, where nvcc is present, for the shapes the reference's GPU kernel
#   handles (see GPU_SHAPES), its exact kernel (cuda.cu:35-253) as device code
#   for sm_103a: oracle/_ref/<shape>/cuda.cubin and the kernel's entry name in
#   oracle/_ref/<shape>/cuda.entry (from ptxas's own report).  The cubin is not
#   x86 code, so it also runs on an Arm host, where the reference sources are absent.
set -euo pipefail
REF=${1:-${BF_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/cpu.cxx" ]; then
  echo "reference sources not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
case "$(uname -m)" in
  x86_64) ARCHFLAG=-march=native ;;
  *) ARCHFLAG=-mcpu=native ;;
esac
CFLAGS="-std=c11 -fopenmp $ARCHFLAG -O3 -DNDEBUG"
CXXFLAGS="-std=c++17 -fopenmp -Drestrict=__restrict__ $ARCHFLAG -O3 -DNDEBUG"

# Shapes T F D P B: the golden-checksum shapes of arraysizes.cxx:54-59, the
# plain-beamform workload, the full single-GPU chunk (t=32768 f=84), the
# wide-array shape (d=1024 b=512), the deepest dish count the tensor-core
# path accepts (d=2048), and small ragged shapes for byte comparison.
SHAPES=${BF_REF_SHAPES:-"
32768 16 512 2 96
32768 32 512 2 96
32768 32 512 2 128
32 32 512 2 128
8 32 512 2 128
1 32 512 2 128
2048 16 512 2 96
64 2 64 2 8
40 3 32 2 16
33 2 48 2 24
8 1 32 2 8
1 1 1 2 1
7 3 5 2 3
16 2 32 1 8
256 1 512 2 128
128 2 1024 2 512
32768 84 512 2 96
16384 16 1024 2 512
64 2 2048 2 96
"}

build_one() {
  local T=$1 F=$2 D=$3 P=$4 B=$5
  local dir="$OUT/${T}_${F}_${D}_${P}_${B}"
  if [ -x "$dir/cpu" ] && [ -x "$dir/ref_io" ]; then return 0; fi
  mkdir -p "$dir"
  sed -E \
    -e "s/^constexpr size_t ntimes = [0-9]+;/constexpr size_t ntimes = ${T};/" \
    -e "s/^constexpr size_t nfrequencies = [0-9]+;/constexpr size_t nfrequencies = ${F};/" \
    -e "s/^constexpr size_t ndishes = [0-9]+;/constexpr size_t ndishes = ${D};/" \
    -e "s/^constexpr size_t npolarizations = [0-9]+;/constexpr size_t npolarizations = ${P};/" \
    -e "s/^constexpr size_t nbeams = [0-9]+;/constexpr size_t nbeams = ${B};/" \
    "$REF/arraysizes.hxx" > "$dir/arraysizes.hxx"
  local inc="-include $dir/arraysizes.hxx -I$REF"
  gcc $CFLAGS -I"$REF" -c "$REF/adler32.c" -o "$dir/adler32.o"
  g++ $CXXFLAGS $inc -c "$REF/arraysizes.cxx" -o "$dir/arraysizes.o"
  g++ $CXXFLAGS $inc -c "$REF/cpu.cxx" -o "$dir/cpu.o"
  g++ $CXXFLAGS -o "$dir/cpu" "$dir/cpu.o" "$dir/arraysizes.o" "$dir/adler32.o"
  g++ $CXXFLAGS $inc -Dmain=reference_stock_main -c "$REF/cpu.cxx" -o "$dir/cpu_lib.o"
  g++ $CXXFLAGS $inc -c "$HERE/ref_io_main.cxx" -o "$dir/ref_io_main.o"
  g++ $CXXFLAGS -o "$dir/ref_io" "$dir/ref_io_main.o" "$dir/cpu_lib.o" "$dir/arraysizes.o" "$dir/adler32.o"
}

# The GPU kernel's launch (cuda.cu:290-296: one block per frequency, 4 x 8 x 12
# threads) covers nbeams only when nbeams / 8 is a multiple of 12 (the assert
# at cuda.cu:76, compiled out by -DNDEBUG; other beam counts would index past
# A and J), so only b = 96 shapes are built: the plain-beamform workload, the
# full single-GPU chunk and a setup()-pattern golden shape.
GPU_SHAPES=${BF_REF_GPU_SHAPES:-"
2048 16 512 2 96
32768 84 512 2 96
32768 16 512 2 96
"}
NVCC=${CUDA_HOME:-/usr/local/cuda}/bin/nvcc
CUFLAGS="-std=c++17 -Drestrict=__restrict__ --expt-relaxed-constexpr -O3 -DNDEBUG -gencode arch=compute_103a,code=sm_103a"

build_gpu() {
  local T=$1 F=$2 D=$3 P=$4 B=$5
  local dir="$OUT/${T}_${F}_${D}_${P}_${B}"
  if [ -f "$dir/cuda.cubin" ] && [ -f "$dir/cuda.entry" ]; then return 0; fi
  [ -f "$dir/arraysizes.hxx" ] || return 1
  "$NVCC" $CUFLAGS -cubin -Xptxas -v -include "$dir/arraysizes.hxx" -I"$REF" "$REF/cuda.cu" \
    -o "$dir/cuda.cubin" 2> "$dir/cuda_ptxas.txt"
  sed -nE "s/.*Compiling entry function '([^']+)'.*/\1/p" "$dir/cuda_ptxas.txt" | head -1 > "$dir/cuda.entry"
  [ -s "$dir/cuda.entry" ]
}

pids=()
while read -r T F D P B; do
  [ -z "${T:-}" ] && continue
  build_one "$T" "$F" "$D" "$P" "$B" &
  pids+=($!)
done <<< "$SHAPES"
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
if [ -x "$NVCC" ]; then
  pids=()
  while read -r T F D P B; do
    [ -z "${T:-}" ] && continue
    build_gpu "$T" "$F" "$D" "$P" "$B" &
    pids+=($!)
  done <<< "$GPU_SHAPES"
  for p in "${pids[@]}"; do wait "$p" || rc=1; done
fi
exit $rc
