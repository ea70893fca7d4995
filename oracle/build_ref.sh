#!/usr/bin/env bash
# Compile lbc's own src/ (read in place, never copied) into oracle/_ref/libref_lbc.so.
# Every public lbc function is renamed with a ref_ prefix by -D so the library can
# be loaded next to the GPU drop-in. Test infrastructure only.
#   usage: oracle/build_ref.sh [LBC_SOURCE_DIR]
# The source directory is the argument, else $LBC_REF, else the read-only lbc
# checkout of the build container below (this recipe is the one place that
# names it). Exit status 2: no lbc sources there (nothing is built). The
# directory used is recorded in oracle/_ref/SOURCE for the tests that compile
# lbc's case mains against this library's headers.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
src="${1:-${LBC_REF:-/root/reference}}"
[ -d "$src/src/core" ] || { echo "lbc sources not found at $src" >&2; exit 2; }
out="$here/_ref"
mkdir -p "$out"
printf '%s\n' "$src" > "$out/SOURCE"
names="main_lbm collision streaming compute_macroscopic_fields compute_force_mem
 mei_initialization sponge_layer bounce_back interpolated_bounce_back
 convective_inlet convective_outlet convective_top convective_bottom
 pressure_inlet pressure_outlet pressure_top pressure_bottom periodic_x periodic_y
 velocity_inlet velocity_outlet velocity_top velocity_bottom
 velocity_inlet_regularized velocity_outlet_regularized velocity_top_regularized
 velocity_bottom_regularized pressure_inlet_regularized pressure_outlet_regularized
 pressure_top_regularized pressure_bottom_regularized write_vtk_binary_2D
 ensure_directory_exists"
defs=""
for n in $names; do defs="$defs -D$n=ref_$n"; done
omp="-fopenmp"
echo 'int main(void){return 0;}' > "$out/omp_probe.c"
gcc -fopenmp "$out/omp_probe.c" -o "$out/omp_probe" 2>/dev/null || omp=""
rm -f "$out/omp_probe.c" "$out/omp_probe"
# -ffp-contract=off: no FMA contraction (gcc contracts by default on aarch64).
gcc -std=gnu99 -O2 -fPIC -shared -w -ffp-contract=off $omp $defs -I"$src/include" \
    "$src"/src/core/*.c "$src"/src/bc/*.c "$src"/src/utils/*.c -lm -o "$out/libref_lbc.so"
echo "built $out/libref_lbc.so"
