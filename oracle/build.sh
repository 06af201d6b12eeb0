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
# lie; only objects and binaries are written, into oracle/_ref/.
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
echo "oracle/build.sh: built oracle/_build and oracle/_ref"
