#!/bin/bash
# Builds oracle/_ref/libqfref.so: the reference's own operator, evaluator and
# learner sources, read in place from the reference checkout and compiled
# unmodified against the project-written headers in oracle/shims (glog,
# gflags, folly, dynamic_bitset, lowest_bit, the configure-generated
# MemoryConfig.hpp, folly::dynamic, boost::split), plus oracle/ref_driver.cpp
# and oracle/ref_loader.cpp (which compiles the reference's main/main.cpp for
# its LoadData).  Test infrastructure only:
# the output is used as a checker (tests/golden/make_golden.py), never by the
# product.  Compiled like the reference's release build (-O3, NDEBUG).
# Without the reference checkout (e.g. on the GPU host) it does nothing.
set -euo pipefail
REF="${QF_REFERENCE:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
# --where prints the reference checkout this script reads and exits (1 when
# its sources are absent), so other checker scripts name no path of their own.
if [ "${1:-}" = "--where" ]; then
  echo "$REF"
  [ -d "$REF/operations" ]
  exit $?
fi
if [ ! -d "$REF/operations" ]; then
  echo "build_ref: no reference sources at $REF; skipped"
  exit 0
fi
mkdir -p "$OUT/obj"
SRCS="operations/RadixPartition operations/BuildHashTable operations/HashJoin operations/Filter
operations/CountAggregator operations/PartitionAssigner operations/LeftSemiJoin
operations/SemiJoinFactory operations/MultiColumnHashJoin storage/FoilHashTable
learner/CandidateLiteralEvaluator learner/CandidateLiteralEnumerator learner/LiteralSelector
learner/QuickFoil learner/QuickFoilTestRunner learner/QuickFoilTimer schema/FoilClause utility/BitVector memory/MemoryUsage
types/Type"
FLAGS="-std=c++14 -O3 -fPIC -DNDEBUG -w -I$HERE/shims -I$REF"
pids=()
for s in $SRCS; do
  g++ $FLAGS -c "$REF/$s.cpp" -o "$OUT/obj/$(echo "$s" | tr / _).o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
# The learner's calls into these two functions are routed through the
# driver's recorders with the linker's --wrap; their mangled names depend on
# the shim types, so they are read from the objects.
EVAL=$(nm "$OUT/obj/learner_CandidateLiteralEvaluator.o" | awk '$2 == "T" && $3 ~ /CandidateLiteralEvaluator8Evaluate/ {print $3}')
EXT=$(nm "$OUT/obj/operations_MultiColumnHashJoin.o" | awk '$2 == "T" && $3 ~ /CreateLabelAwareBindingTables/ {print $3}')
SELECT=$(nm "$OUT/obj/operations_SemiJoinFactory.o" | awk '$2 == "T" && $3 ~ /SelectAndCreateSemiJoin/ {print $3}')
CREATE=$(nm "$OUT/obj/operations_SemiJoinFactory.o" | awk '$2 == "T" && $3 ~ /14CreateSemiJoin/ {print $3}')
AFTER=$(nm "$OUT/obj/operations_BuildHashTable.o" | awk '$2 == "T" && $3 ~ /BuildHashTableAfterSemiJoin/ {print $3}')
printf '#define QFREF_EVALUATE "%s"\n#define QFREF_EXTEND "%s"\n#define QFREF_SELECT "%s"\n#define QFREF_CREATE "%s"\n#define QFREF_AFTER "%s"\n' \
  "$EVAL" "$EXT" "$SELECT" "$CREATE" "$AFTER" > "$OUT/wrap_names.h"
g++ $FLAGS -I"$OUT" -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
p1=$!
g++ $FLAGS -c "$HERE/ref_loader.cpp" -o "$OUT/obj/ref_loader.o" &
p2=$!
wait "$p1"
wait "$p2"
g++ -shared -o "$OUT/libqfref.so.tmp" "$OUT"/obj/*.o "-Wl,--wrap=$EVAL" "-Wl,--wrap=$EXT" \
  "-Wl,--wrap=$SELECT" "-Wl,--wrap=$CREATE" "-Wl,--wrap=$AFTER"
mv "$OUT/libqfref.so.tmp" "$OUT/libqfref.so"
echo "build_ref: $OUT/libqfref.so"
