#!/usr/bin/env bash
# Builds the MDACP reference from its own sources, in place, for use as an
# oracle and CPU baseline (test infrastructure only).  Outputs go to
# oracle/_ref/ only; nothing from the reference is committed.
#
#   MDG_REFERENCE_DIR   reference source directory (default /root/reference)
#   MDG_REF_N           per-unit particle capacity N (mdconfig.h:11), default 1000000
#
# The reference fixes the cut-off at compile time (mdconfig.h:15,
# CUTOFF_LENGTH = 3.0).  For each cut-off built here a copy of mdconfig.h with
# that value (and capacity N) is generated under oracle/_ref/gen/ and
# force-included; its include guard makes every later #include "mdconfig.h"
# from the reference sources a no-op.  The single-rank MPI stand-in is
# oracle/mpi_shim/mpi.h.  -std=c++17 is needed for the aligned(64) members of
# Variables; -ffp-contract=off keeps the arithmetic free of fused multiply-adds
# (the reference's default x86-64 build has none).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${MDG_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
N="${MDG_REF_N:-1000000}"
if [ ! -f "$REF/mdconfig.h" ]; then
  echo "reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/gen"
SRCS=$(ls "$REF"/*.cc)
build_one() {
  local rc="$1" tag="$2"
  local gen="$OUT/gen/mdconfig_$tag.h"
  sed -e "s/^const double CUTOFF_LENGTH = 3.0;/const double CUTOFF_LENGTH = $rc;/" \
      -e "s/^const int N = 1000000;/const int N = $N;/" "$REF/mdconfig.h" > "$gen"
  grep -q "CUTOFF_LENGTH = $rc;" "$gen"
  g++ -O3 -std=c++17 -fopenmp -ffp-contract=off -w \
      -include "$gen" -I "$HERE/mpi_shim" -I "$REF" \
      $SRCS "$HERE/ref_harness.cc" -o "$OUT/mdacp_$tag"
}
build_one 2.5 rc2.5 &
build_one 3.0 rc3.0 &
wait
echo "built: $(ls "$OUT"/mdacp_*)"
