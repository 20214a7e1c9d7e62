#!/usr/bin/env bash
# Build recipe for the oracle (test infrastructure only).
#
#   oracle/_build/libheat_oracle.so   the C restatement (heat_ref.c) for ctypes
#   oracle/_build/heat_ref            its command-line front end
#   oracle/_ref/serial                the UNMODIFIED reference serial solver,
#                                     compiled from its own source where it lies
#   oracle/_ref/src/1-cuda.cu         the reference's single-GPU CUDA program,
#                                     staged (copied unmodified, git-ignored) so
#                                     that it can be built on a GPU machine
#   oracle/_ref/1-cuda                that program built for sm_103a with the
#                                     reference Makefile's flags (CUDA/Makefile:
#                                     36-37; only -arch changed), where nvcc is
#
# The reference checkout is looked for in $HEAT_REFERENCE_ROOT, else beside
# this repository (../reference); without it only the restatement is built
# (and a previously staged 1-cuda.cu is still compiled).
#
# Flags follow the reference serial build
# (3D_Heat_Benchmark/NVIDIA-H100/Source-Results/OpenMP/Makefile:23):
# -O3 -fopenmp -ffp-contract=off -lm.  The reference's own build system is not
# run; the serial is a single self-contained C file, and so is 1-cuda.cu.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
PKG="$ROOT/openmp-offloading-intranode-artifact_gb300"
REF_ROOT="${HEAT_REFERENCE_ROOT:-$ROOT/../reference}"
REF_SRC="$REF_ROOT/OpenMP_Single_Source/heat3D_variable_coeff.c"
REF_CUDA1="$REF_ROOT/3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/1-cuda.cu"
CC="${CC:-gcc}"
CXX="${CXX:-g++}"
FLAGS="-O3 -fopenmp -ffp-contract=off"

mkdir -p "$HERE/_build"
# Host-only input generator shared with the library (no CUDA involved).
$CXX $FLAGS -fPIC -std=c++17 -I"$ROOT/include" -c "$PKG/csrc/heat_inputs.cpp" -o "$HERE/_build/heat_inputs.o"
$CC $FLAGS -fPIC -std=c11 -D_DEFAULT_SOURCE -I"$ROOT/include" -I"$HERE" -c "$HERE/heat_ref.c" -o "$HERE/_build/heat_ref.o"
$CC $FLAGS -std=c11 -D_DEFAULT_SOURCE -I"$ROOT/include" -I"$HERE" -c "$HERE/heat_ref_main.c" -o "$HERE/_build/heat_ref_main.o"
$CXX $FLAGS -shared -o "$HERE/_build/libheat_oracle.so" "$HERE/_build/heat_ref.o" "$HERE/_build/heat_inputs.o" -lm
$CXX $FLAGS -o "$HERE/_build/heat_ref" "$HERE/_build/heat_ref_main.o" "$HERE/_build/heat_ref.o" "$HERE/_build/heat_inputs.o" -lm

if [[ -f "$REF_SRC" ]]; then
  mkdir -p "$HERE/_ref"
  $CC $FLAGS -o "$HERE/_ref/serial" "$REF_SRC" -lm
  echo "built oracle/_ref/serial from the reference serial"
else
  echo "reference serial source not present; oracle/_ref/serial not rebuilt"
fi

if [[ -f "$REF_CUDA1" ]]; then
  mkdir -p "$HERE/_ref/src"
  install -m 0644 "$REF_CUDA1" "$HERE/_ref/src/1-cuda.cu"
fi
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
if [[ -f "$HERE/_ref/src/1-cuda.cu" && -x "$NVCC" ]]; then
  if "$NVCC" -O3 --fmad=false --prec-div=true --prec-sqrt=true --ftz=false -arch=sm_103a \
       -Xcompiler -fopenmp -o "$HERE/_ref/1-cuda" "$HERE/_ref/src/1-cuda.cu" -lm; then
    echo "built oracle/_ref/1-cuda (reference 1-cuda.cu, sm_103a)"
  else
    echo "reference 1-cuda.cu did not build; oracle/_ref/1-cuda absent"
    rm -f "$HERE/_ref/1-cuda"
  fi
fi
echo "built oracle/_build/{libheat_oracle.so,heat_ref}"
