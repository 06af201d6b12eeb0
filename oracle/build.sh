#!/bin/sh
# TEST INFRASTRUCTURE build recipe for the checker side (never the product).
#
#   oracle/_build/liboracle.so   the C restatement (flowshop_oracle.c)
#   oracle/_ref/libref_bound.so  the reference's own bound_flowshop, compiled
#   oracle/_ref/ref_explore      in place from the reference tree, plus the
#                                harnesses in oracle/ref_harness/
#
# The reference part runs only where the reference tree exists (this build
# container); elsewhere it is skipped. Reference sources are read where they
# lie; only objects and binaries are written, into oracle/_ref/. The tree is
# taken from WSBB_REFERENCE_DIR, else from the one default location below;
# the location used is recorded in oracle/_ref/reference_dir, which is how
# the tests find it (nothing else names a path of the reference).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${WSBB_REFERENCE_DIR:-/root/reference}
CC=${CC:-gcc}
CXX=${CXX:-g++}

mkdir -p "$HERE/_build"
$CC -O2 -fPIC -shared -std=gnu11 -Wall -Wno-unused-function \
    -o "$HERE/_build/liboracle.so" "$HERE/flowshop_oracle.c" -lpthread

if [ ! -d "$REF/src" ]; then
	echo "oracle/build.sh: no reference tree at $REF; oracle/_ref skipped"
	exit 0
fi

OBJ="$HERE/_ref/obj"
mkdir -p "$OBJ"
printf '%s\n' "$REF" > "$HERE/_ref/reference_dir"
INC="-I$HERE/ref_shim/src -I$HERE/ref_shim/headers -I$REF/headers"
# The reference targets pre-C++11 compilers (solutions.cpp:30 compares an
# ifstream with NULL), so it is compiled as gnu++98; warnings are its own.
CXXREF="$CXX -std=gnu++98 -O2 -fPIC -w $INC"

for f in bound_flowshop bound_abstract tree decompose_beginend problems \
         bb_problem_calculator select_worst solutions eliminate_pareto \
         weights work peer ttime instance_flowshop; do
	$CXXREF -c "$REF/src/$f.cpp" -o "$OBJ/$f.o"
done
for f in BigInteger BigUnsigned BigIntegerUtils BigUnsignedInABase; do
	$CXXREF -c "$REF/int/$f.cc" -o "$OBJ/$f.o"
done

$CXXREF -c "$HERE/ref_harness/ref_bound.cpp" -o "$OBJ/ref_bound.o"
$CXXREF -c "$HERE/ref_harness/ref_explore.cpp" -o "$OBJ/ref_explore.o"
$CXXREF -c "$HERE/ref_harness/ref_gen.cpp" -o "$OBJ/ref_gen.o"

$CXX -shared -o "$HERE/_ref/libref_bound.so" "$OBJ/ref_bound.o" "$OBJ/ref_gen.o" \
    "$OBJ/bound_flowshop.o" "$OBJ/bound_abstract.o" "$OBJ/instance_flowshop.o" -lpthread

$CXX -o "$HERE/_ref/ref_explore" "$OBJ/ref_explore.o" \
    "$OBJ/bound_flowshop.o" "$OBJ/bound_abstract.o" "$OBJ/tree.o" \
    "$OBJ/decompose_beginend.o" "$OBJ/problems.o" \
    "$OBJ/bb_problem_calculator.o" "$OBJ/select_worst.o" \
    "$OBJ/solutions.o" "$OBJ/eliminate_pareto.o" "$OBJ/weights.o" \
    "$OBJ/work.o" "$OBJ/peer.o" "$OBJ/ttime.o" "$OBJ/instance_flowshop.o" \
    "$OBJ/BigInteger.o" "$OBJ/BigUnsigned.o" "$OBJ/BigIntegerUtils.o" \
    "$OBJ/BigUnsignedInABase.o" -lpthread
# The same search for n up to 64. The reference caps n at MAX_NBJOBS = 20
# (headers/tree.h:31, headers/explorer.h:34: the rank-path comparator and
# the node record are sized by it), so a copy of its sources with that one
# constant raised to 64 is made under oracle/_ref/big/ (a build directory,
# never committed) and compiled the same way into oracle/_ref/ref_explore_big.
# The copy is needed because the sources include their headers by relative
# path ("../headers/tree.h"), which no include flag can redirect.
BIG="$HERE/_ref/big"
rm -rf "$BIG"
mkdir -p "$BIG/src" "$HERE/_ref/objbig"
cp -r "$REF/headers" "$REF/int" "$BIG/"
for f in bound_flowshop bound_abstract tree decompose_beginend problems \
         bb_problem_calculator select_worst solutions eliminate_pareto \
         weights work peer ttime instance_flowshop; do
	cp "$REF/src/$f.cpp" "$BIG/src/"
done
sed -i 's/^#define MAX_NBJOBS 20$/#define MAX_NBJOBS 64/' "$BIG/headers/tree.h" "$BIG/headers/explorer.h"
grep -q '^#define MAX_NBJOBS 64$' "$BIG/headers/tree.h"
grep -q '^#define MAX_NBJOBS 64$' "$BIG/headers/explorer.h"
OBJB="$HERE/_ref/objbig"
CXXBIG="$CXX -std=gnu++98 -O2 -fPIC -w -DWSBB_SHIM_MAXJOBS=64 -I$HERE/ref_shim/src -I$HERE/ref_shim/headers -I$BIG/headers"
BOBJS=""
for f in bound_flowshop bound_abstract tree decompose_beginend problems \
         bb_problem_calculator select_worst solutions eliminate_pareto \
         weights work peer ttime instance_flowshop; do
	$CXXBIG -c "$BIG/src/$f.cpp" -o "$OBJB/$f.o" &
	BOBJS="$BOBJS $OBJB/$f.o"
done
for f in BigInteger BigUnsigned BigIntegerUtils BigUnsignedInABase; do
	$CXXBIG -c "$BIG/int/$f.cc" -o "$OBJB/$f.o" &
	BOBJS="$BOBJS $OBJB/$f.o"
done
$CXXBIG -c "$HERE/ref_harness/ref_explore.cpp" -o "$OBJB/ref_explore.o" &
wait
$CXX -o "$HERE/_ref/ref_explore_big" "$OBJB/ref_explore.o" $BOBJS -lpthread
rm -rf "$BIG" "$OBJB"   # the copy only served this build
echo "oracle/build.sh: built oracle/_build and oracle/_ref"
