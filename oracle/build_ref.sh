#!/usr/bin/env bash
# Build recipe for the oracle (test infrastructure only).
#
#   oracle/_build/libheat_oracle.so   the C restatement (heat_ref.c) for ctypes
#   oracle/_build/heat_ref            its command-line front end
#   oracle/_ref/serial                the UNMODIFIED reference serial solver,
#                                     compiled from its own source where it lies
#                                     (only when the reference tree is present)
#
# Flags follow the reference serial build
# (3D_Heat_Benchmark/NVIDIA-H100/Source-Results/OpenMP/Makefile:23):
# -O3 -fopenmp -ffp-contract=off -lm.  The reference's own build system is not
# run; the serial is a single self-contained C file.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
PKG="$ROOT/openmp-offloading-intranode-artifact_gb300"
REF_SRC="${HEAT_REFERENCE_SRC:-/root/reference/OpenMP_Single_Source/heat3D_variable_coeff.c}"
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
  echo "built oracle/_ref/serial from $REF_SRC"
else
  echo "reference source not present; oracle/_ref not rebuilt"
fi
echo "built oracle/_build/{libheat_oracle.so,heat_ref}"
