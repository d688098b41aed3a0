#!/bin/sh
# Stage the reference's CUDA headers (chabner/temporalSpecklesCode) for the
# harness build: copies the header tree from a reference checkout into
# oracle/_ref/src, which git ignores (the reference's sources are never part
# of this repository).  The harness itself is built where a GPU runs it:
#   sh oracle/stage_reference.sh /path/to/temporalSpecklesCode
#   make -C oracle -f refharness.mk
set -e
if [ $# -ne 1 ]; then
    echo "usage: sh oracle/stage_reference.sh <root of the reference checkout>" >&2
    exit 2
fi
ref="$1"
here="$(cd "$(dirname "$0")" && pwd)"
dst="$here/_ref/src"
mkdir -p "$dst/Interface" "$dst/Implementation/Medium" "$dst/Implementation/Sampler" "$dst/Implementation/Source" "$dst/Implementation/Tracer"
for f in Simulation.cuh ComplexType.cuh VectorType.cuh MatrixOperations.cuh SpecialFunctions.cuh; do
    cp "$ref/$f" "$dst/$f"
done
cp "$ref"/Interface/*.cuh "$dst/Interface/"
cp "$ref"/Implementation/Scattering.cuh "$dst/Implementation/"
for d in Medium Sampler Source Tracer; do
    cp "$ref"/Implementation/$d/*.cuh "$dst/Implementation/$d/"
done
echo "staged the reference headers in $dst"
