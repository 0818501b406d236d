#!/bin/sh
# Builds the reference-derived test programs from the reference sources where they
# lie.  Outputs go only into oracle/_ref/ (git-ignored).  Needs the reference
# tree ($REF, else the directory `reference` beside this repository); without
# it this script does nothing.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-$HERE/../../../reference}
OUT="$HERE/../_ref"
if [ ! -d "$REF/cuda/pagani/quad" ]; then
  echo "build_ref: reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
# Host-only dumper of the reference's rule tables (x86 host of this container).
$NVCC -std=c++17 --expt-relaxed-constexpr -w -I"$REF" -I"$REF/externals" \
  -o "$OUT/dump_rule_tables" "$HERE/dump_rule_tables.cu"
# Reference evaluation kernel for sm_103a as a cubin (loaded on the GPU machine
# through the driver API; no host code of the reference is needed there).
if [ -f "$HERE/ref_phase1.cu" ]; then
  $NVCC -std=c++17 --expt-relaxed-constexpr -w -I"$REF" -I"$REF/externals" -I"$HERE/../.." \
    -gencode arch=compute_103a,code=sm_103a -cubin -o "$OUT/ref_phase1.cubin" "$HERE/ref_phase1.cu"
fi
# Reference two-level, filter and split kernels as a cubin (same loading path).
if [ -f "$HERE/ref_stages.cu" ]; then
  $NVCC -std=c++17 --expt-relaxed-constexpr -w -I"$REF" -I"$REF/externals" \
    -gencode arch=compute_103a,code=sm_103a -cubin -o "$OUT/ref_stages.cubin" "$HERE/ref_stages.cu"
fi
# The reference's m-Cubes sampling kernels as a cubin.
if [ -f "$HERE/ref_mcubes.cu" ]; then
  $NVCC -std=c++17 --expt-relaxed-constexpr -w -I"$REF" -I"$REF/externals" -I"$HERE/../.." \
    -gencode arch=compute_103a,code=sm_103a -cubin -o "$OUT/ref_mcubes.cubin" "$HERE/ref_mcubes.cu"
fi
# The reference's sequential CPU m-Cubes (host program of this container).
if [ -f "$HERE/mcubes_seq_run.cu" ]; then
  $NVCC -std=c++17 --expt-relaxed-constexpr -w -O2 -I"$REF" -I"$REF/externals" \
    -o "$OUT/mcubes_seq_run" "$HERE/mcubes_seq_run.cu"
fi
echo "build_ref: done -> $OUT"
