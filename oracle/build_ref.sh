#!/usr/bin/env bash
# Compile the reference's own driver sources (src/main.cpp and include/, read
# in place, unmodified) against the project's Kokkos-API shim into
# oracle/_ref/libkpt_ref.so.  Test infrastructure: used to make golden vectors
# and to pin the oracle restatement.  Needs the reference checkout; a machine
# without it skips this step.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${KPT_REFERENCE_DIR:-/root/reference}"
if [ ! -f "$ref/src/main.cpp" ]; then
    echo "build_ref: reference sources not found at $ref; skipping" >&2
    exit 0
fi
mkdir -p "$here/_ref"
# libkpt_ref.so: Kokkos::pow is the project pow (bit-for-bit parity with the
# GPU and the restatement); libkpt_ref_libm.so: the C library's pow, as a real
# Kokkos host build calls (timed against the restatement's libm build)
build() {
    g++ -O2 -std=c++20 -fopenmp -ffp-contract=off -fPIC -shared \
        -Dmain=kpt_ref_main "$@" \
        -I "$here/kokkos_shim" -I "$here/../kokkos-particletransport_gb300/csrc" \
        -I "$ref" -I "$ref/include" \
        "$here/ref_harness.cpp" -o "$out.tmp"
    mv "$out.tmp" "$out"
    echo "build_ref: wrote $out"
}
out="$here/_ref/libkpt_ref.so" build & first=$!
out="$here/_ref/libkpt_ref_libm.so" build -DKPT_SHIM_LIBM_POW & second=$!
wait "$first"
wait "$second"
