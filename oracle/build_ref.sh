#!/usr/bin/env bash
# Compiles the reference's exact-diagonalization sources (spinless, then spinful), unmodified
# and in place under the read-only reference checkout, into the probe
# oracle/_ref/ref_probe (test infrastructure; outputs go to oracle/_ref only).
#
# Needs: g++, the reference checkout, and scipy's bundled OpenBLAS for the two
# LAPACK calls (oracle/shim/lapack_shim.c). The GSL headers the reference
# includes are replaced by stand-ins (oracle/shim/gsl); no GSL routine runs.
#
# Flags follow the reference Makefile's link line (-O2 -fopenmp), applied at
# compile time as well so that the OpenMP loops of matrix.cpp are active.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${BLQH_REFERENCE:-/root/reference}/BLQH_without_spin"
OUT="$HERE/_ref"
if [ ! -d "$REF" ]; then echo "build_ref.sh: no reference checkout at $REF" >&2; exit 3; fi
BLAS_DIR="$(python3 -c 'import scipy, os; print(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs"))')"
BLAS_LIB="$(ls "$BLAS_DIR"/libscipy_openblas*.so | head -1)"
mkdir -p "$OUT"
CXXFLAGS="-std=c++11 -O2 -fopenmp -w -I$HERE/shim -I$REF"
for f in basis matrix lanczos_hamiltonian hamiltonian; do
  g++ $CXXFLAGS -c "$REF/$f.cpp" -o "$OUT/$f.o" &
done
g++ $CXXFLAGS -c "$HERE/ref_probe.cpp" -o "$OUT/ref_probe.o" &
g++ $CXXFLAGS -c "$HERE/ref_saveload.cpp" -o "$OUT/ref_saveload.o" &
gcc -O2 -I"$HERE/shim" -c "$HERE/shim/gsl_stub.c" -o "$OUT/gsl_stub.o" &
gcc -O2 -c "$HERE/shim/lapack_shim.c" -o "$OUT/lapack_shim.o" &
wait
g++ -O2 -fopenmp -o "$OUT/ref_probe" "$OUT"/ref_probe.o "$OUT"/basis.o "$OUT"/matrix.o \
  "$OUT"/lanczos_hamiltonian.o "$OUT"/hamiltonian.o "$OUT"/gsl_stub.o "$OUT"/lapack_shim.o \
  "$BLAS_LIB" -Wl,-rpath,"$BLAS_DIR" -lpthread
echo "built $OUT/ref_probe"
g++ -O2 -fopenmp -o "$OUT/ref_saveload" "$OUT"/ref_saveload.o "$OUT"/basis.o "$OUT"/matrix.o \
  "$OUT"/lanczos_hamiltonian.o "$OUT"/hamiltonian.o "$OUT"/gsl_stub.o "$OUT"/lapack_shim.o \
  "$BLAS_LIB" -Wl,-rpath,"$BLAS_DIR" -lpthread
echo "built $OUT/ref_saveload"

# The spinful model (BLQH_with_spin), the same way, into oracle/_ref/spin.
REFS="${BLQH_REFERENCE:-/root/reference}/BLQH_with_spin"
OUTS="$OUT/spin"
if [ -d "$REFS" ]; then
  mkdir -p "$OUTS"
  CXXS="-std=c++11 -O2 -fopenmp -w -I$HERE/shim -I$REFS"
  for f in basis matrix lanczos_hamiltonian hamiltonian; do
    g++ $CXXS -c "$REFS/$f.cpp" -o "$OUTS/$f.o" &
  done
  g++ $CXXS -c "$HERE/ref_probe_spin.cpp" -o "$OUTS/ref_probe_spin.o" &
  wait
  g++ -O2 -fopenmp -o "$OUT/ref_probe_spin" "$OUTS"/ref_probe_spin.o "$OUTS"/basis.o "$OUTS"/matrix.o \
    "$OUTS"/lanczos_hamiltonian.o "$OUTS"/hamiltonian.o "$OUT"/gsl_stub.o "$OUT"/lapack_shim.o \
    "$BLAS_LIB" -Wl,-rpath,"$BLAS_DIR" -lpthread
  echo "built $OUT/ref_probe_spin"
fi

# The reference's Makefile compiles with -std=c++11 only (no optimization, no
# OpenMP at compile time): BLQH_REF_O0=1 also builds that variant of the probe,
# oracle/_ref/ref_probe_O0, to time the reference as it ships.
if [ "${BLQH_REF_O0:-0}" = "1" ]; then
  OUT0="$OUT/O0"
  mkdir -p "$OUT0"
  for f in basis matrix lanczos_hamiltonian hamiltonian; do
    g++ -std=c++11 -w -I"$HERE/shim" -I"$REF" -c "$REF/$f.cpp" -o "$OUT0/$f.o" &
  done
  g++ -std=c++11 -w -I"$HERE/shim" -I"$REF" -c "$HERE/ref_probe.cpp" -o "$OUT0/ref_probe.o" &
  wait
  g++ -fopenmp -o "$OUT/ref_probe_O0" "$OUT0"/ref_probe.o "$OUT0"/basis.o "$OUT0"/matrix.o \
    "$OUT0"/lanczos_hamiltonian.o "$OUT0"/hamiltonian.o "$OUT"/gsl_stub.o "$OUT"/lapack_shim.o \
    "$BLAS_LIB" -Wl,-rpath,"$BLAS_DIR" -lpthread
  echo "built $OUT/ref_probe_O0"
fi
