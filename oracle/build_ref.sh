#!/usr/bin/env bash
# TEST INFRASTRUCTURE (oracle).  Builds the UNMODIFIED SpatialPy C++ engine
# from its sources where they lie under the reference package, together with
# oracle/ref_driver.cpp, into oracle/_ref/ (git-ignored):
#   libspref.so        stock engine (-O2)
#   libspref_exact.so  the exact SSA that SP_SELECT_EXACT runs: the same
#                      engine with the two selection lines of
#                      src/simulate_rdme.cpp:260,317 rescaled, no event past
#                      the step end (the loop of :233-238 returns when the
#                      selected time lies beyond it; selectReaction only
#                      peeks), and a diffusion destination's reactions
#                      evaluated with its own volume (:431-433) (a patched
#                      copy written into oracle/_ref/, never into the
#                      repository)
#   libspref_O0.so     stock engine at -O0, as the shipped SCons build compiles it
# File lists follow src/SConscript:2-12 and external/ANN/src/SConscript:2-17.
# -ftrivial-auto-var-init=zero makes the engine's uninitialised step-0 particle
# fields deterministic (particle.cpp:70-83).  Needs g++ only (no SCons).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
# the reference checkout, or its pip install in baseline/_ref (same layout)
ref="${SPATIALPY_REFERENCE:-$here/../baseline/_ref}"
eng="$ref/spatialpy/solvers/c_base/ssa_sdpd-c-simulation-engine"
out="$here/_ref"
if [ ! -d "$eng/src" ]; then
  echo "reference engine sources not found under $eng" >&2
  exit 2
fi
mkdir -p "$out"
# nothing to do when every library is newer than the driver, this recipe and the ABI header
stale=0
for v in "" _exact _O0; do
  lib="$out/libspref$v.so"
  if [ ! -f "$lib" ] || [ "$here/ref_driver.cpp" -nt "$lib" ] || [ "$0" -nt "$lib" ] ||
     [ "$here/../include/spgpu.h" -nt "$lib" ]; then stale=1; fi
done
if [ "$stale" = 0 ] && [ "${1:-}" != "--force" ]; then
  echo "up to date: $(ls "$out"/*.so | xargs -n1 basename | tr '\n' ' ')"
  exit 0
fi
core="count_cores model NRMConstant_v5 output particle pthread_barrier simulate simulate_threads"
ann="ANN brute kd_tree kd_util kd_split kd_dump kd_search kd_pr_search kd_fix_rad_search bd_tree bd_search bd_pr_search bd_fix_rad_search perf"
inc="-I$eng/include -I$eng/external/ANN/include -I$here/../include"

build_variant() {  # $1 = suffix, $2 = optimisation flag, $3 = simulate_rdme source
  local sfx="$1" opt="$2" rdme="$3" objs=() pids=()
  local flags="-std=c++14 $opt -fPIC -ftrivial-auto-var-init=zero -ffp-contract=off -w"
  for f in $core; do
    g++ $flags $inc -c "$eng/src/$f.cpp" -o "$out/$f$sfx.o" & pids+=($!)
    objs+=("$out/$f$sfx.o")
  done
  for f in $ann; do
    g++ $flags $inc -c "$eng/external/ANN/src/$f.cpp" -o "$out/ann_$f$sfx.o" & pids+=($!)
    objs+=("$out/ann_$f$sfx.o")
  done
  g++ $flags $inc -c "$rdme" -o "$out/simulate_rdme$sfx.o" & pids+=($!)
  objs+=("$out/simulate_rdme$sfx.o")
  g++ $flags $inc -c "$here/ref_driver.cpp" -o "$out/ref_driver$sfx.o" & pids+=($!)
  objs+=("$out/ref_driver$sfx.o")
  for p in "${pids[@]}"; do wait "$p"; done
  g++ -shared -o "$out/libspref$sfx.so" "${objs[@]}" -lpthread
}

# exact-selection twin: rescale the reused uniform (rand1) to the chosen class
sed -e 's/double rand_rval = rand1 \* subvol->srrate;/double rand_rval = rand1 * totrate;/' \
    -e 's/double diff_rand = rand1 \* subvol->sdrate;/double diff_rand = rand1 * totrate - subvol->srrate;/' \
    -e 's|(dest_subvol->xx,tt,vol,dest_subvol->data_fn,dest_subvol->type)|(dest_subvol->xx,tt,dest_subvol->mass / dest_subvol->rho,dest_subvol->data_fn,dest_subvol->type)|' \
    -e 's|subvol_index = timeRxnPair.second;|subvol_index = timeRxnPair.second; if (tt > end_time) return;|' \
    "$eng/src/simulate_rdme.cpp" > "$out/simulate_rdme_exact.cpp"
grep -q 'rand_rval = rand1 \* totrate' "$out/simulate_rdme_exact.cpp"
grep -q 'diff_rand = rand1 \* totrate - subvol->srrate' "$out/simulate_rdme_exact.cpp"
grep -q '(dest_subvol->xx,tt,dest_subvol->mass / dest_subvol->rho,' "$out/simulate_rdme_exact.cpp"
grep -q 'subvol_index = timeRxnPair.second; if (tt > end_time) return;' "$out/simulate_rdme_exact.cpp"

build_variant "" "-O2" "$eng/src/simulate_rdme.cpp"
build_variant "_exact" "-O2" "$out/simulate_rdme_exact.cpp"
build_variant "_O0" "-O0" "$eng/src/simulate_rdme.cpp"
rm -f "$out"/*.o
echo "built: $(ls "$out"/*.so | xargs -n1 basename | tr '\n' ' ')"
