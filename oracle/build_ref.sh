#!/usr/bin/env bash
# Builds the unmodified meso-lts solver sources into oracle/_ref/meso_ref.
#
# Test infrastructure only: the binary is the reference itself, used to pin
# the C restatement in oracle/ and to generate tests/golden/ fixtures.  It is
# built from the sources where they lie, in the checkout that $MESO_REF_SRC
# names (required); nothing is copied into the repository.  Outputs go to
# oracle/_ref/ (git-ignored).
#
#   MESO_REF_SRC=<meso-lts checkout> bash oracle/build_ref.sh
#
# Substitutions, all project-written:
#   * oracle/ref/mpi.h        single-rank MPI (the image has no MPI library)
#   * oracle/ref/metis_stub.cpp   METIS entry points (only the out-of-scope
#                                 --mesh partition path calls them)
#   * field.cpp is compiled from a patched copy written into oracle/_ref/:
#     GatherFieldList (src/solver/field.cpp:203-205) reads displacements[-1]
#     at i = 0; the copy starts that loop at i = 1.  Only symmetry and
#     slip-wall faces call it.
# Flags: -O2 -ffp-contract=off, so no FMA contraction on any host.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ -z "${MESO_REF_SRC:-}" ]; then
    echo "MESO_REF_SRC is not set: name the meso-lts checkout to build oracle/_ref from" >&2
    exit 2
fi
SRC="$MESO_REF_SRC"
OUT="$HERE/_ref"
if [ ! -d "$SRC/src" ]; then
    echo "reference sources not found at $SRC; skipping oracle/_ref build" >&2
    exit 0
fi
mkdir -p "$OUT/obj"
sed '203s/int i = 0;/int i = 1;/' "$SRC/src/solver/field.cpp" > "$OUT/field_patched.cpp"
grep -q 'for (int i = 1; i < MPI::processor_num' "$OUT/field_patched.cpp"

CXX="${CXX:-g++}"
FLAGS=(-O2 -std=c++17 -ffp-contract=off -w -I"$HERE/ref" -I"$SRC/include")
srcs=()
while IFS= read -r f; do
    case "$f" in
        */src/meso/main.cpp|*/src/solver/field.cpp) ;;
        *) srcs+=("$f") ;;
    esac
done < <(find "$SRC/src" -name '*.cpp' | sort)
srcs+=("$OUT/field_patched.cpp" "$HERE/ref/metis_stub.cpp" "$HERE/ref/harness.cpp")

pids=()
objs=()
for f in "${srcs[@]}"; do
    o="$OUT/obj/$(echo "$f" | sed 's#[/.]#_#g').o"
    objs+=("$o")
    if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
        "$CXX" "${FLAGS[@]}" -c "$f" -o "$o" &
        pids+=($!)
    fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -O2 -o "$OUT/meso_ref" "${objs[@]}"
echo "built $OUT/meso_ref"
