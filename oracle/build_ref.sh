#!/usr/bin/env bash
# Builds the MDACP reference from its own sources, for use as an oracle and
# as the timed CPU baseline (test infrastructure only).  Outputs go to
# oracle/_ref/ only (git-ignored); nothing from the reference is committed.
#
#   MDG_REFERENCE_DIR   reference source directory.  When set, its sources
#                       (*.cc, *.h) are first staged into oracle/_ref/src/, so
#                       that a copy of this tree on another machine (without
#                       the reference) can rebuild the binaries from there.
#                       When unset, oracle/_ref/src/ must already hold them.
#   MDG_REF_N           per-unit particle capacity N (mdconfig.h:11), default 1000000
#
# The reference fixes the cut-off at compile time (mdconfig.h:15,
# CUTOFF_LENGTH = 3.0).  For each cut-off built here a copy of mdconfig.h with
# that value (and capacity N) is generated under oracle/_ref/gen/ and
# force-included; its include guard makes every later #include "mdconfig.h"
# from the reference sources a no-op.  The single-rank MPI stand-in is
# oracle/mpi_shim/mpi.h.  -std=c++17 is needed for the aligned(64) members of
# Variables.
#
# Two kinds of binary:
#   mdacp_rc<rc>        parity binaries: -ffp-contract=off keeps the
#                       arithmetic free of fused multiply-adds (the
#                       reference's default x86-64 build has none), so the
#                       oracle can be pinned to them bit for bit;
#   mdacp_bench_rc2.5   the timed CPU baseline: -O3 with the compiler's default
#                       contraction (fused multiply-adds where the target has
#                       them), as the reference's own makefile builds it.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
N="${MDG_REF_N:-1000000}"
if [ -n "${MDG_REFERENCE_DIR:-}" ]; then
  if [ ! -f "$MDG_REFERENCE_DIR/mdconfig.h" ]; then
    echo "reference sources not found at $MDG_REFERENCE_DIR" >&2
    exit 3
  fi
  mkdir -p "$SRC"
  cp "$MDG_REFERENCE_DIR"/*.cc "$MDG_REFERENCE_DIR"/*.h "$SRC"/
fi
if [ ! -f "$SRC/mdconfig.h" ]; then
  echo "no reference sources: set MDG_REFERENCE_DIR" >&2
  exit 3
fi
mkdir -p "$OUT/gen"
SRCS=$(ls "$SRC"/*.cc)
build_one() {
  local rc="$1" tag="$2" flags="$3"
  local gen="$OUT/gen/mdconfig_$tag.h"
  sed -e "s/^const double CUTOFF_LENGTH = 3.0;/const double CUTOFF_LENGTH = $rc;/" \
      -e "s/^const int N = 1000000;/const int N = $N;/" "$SRC/mdconfig.h" > "$gen"
  grep -q "CUTOFF_LENGTH = $rc;" "$gen"
  g++ -O3 -std=c++17 -fopenmp $flags -w \
      -include "$gen" -I "$HERE/mpi_shim" -I "$SRC" \
      $SRCS "$HERE/ref_harness.cc" -o "$OUT/mdacp_$tag.tmp$$"
  mv "$OUT/mdacp_$tag.tmp$$" "$OUT/mdacp_$tag"
}
build_one 2.5 rc2.5 -ffp-contract=off &
build_one 3.0 rc3.0 -ffp-contract=off &
build_one 2.5 bench_rc2.5 "" &
wait
echo "built: $(ls "$OUT"/mdacp_*)"
