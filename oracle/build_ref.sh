#!/usr/bin/env bash
# Builds the parity checker from the UNMODIFIED dCNS reference sources where they lie (read-only checkout),
# plus oracle/ref_harness.cpp, into oracle/_ref/libdcns_ref.so.  Test infrastructure only.
#
#   -include cstdint : model/Matrix.cpp uses int32_t without including <cstdint> (GCC 13 rejects it otherwise)
#   -mavx2           : selects the reference's AVX2 SmithWaterman (impl/sequenceAlignment3.cpp:223), the path its
#                      shipped x86 binary runs; on a non-x86 host the scalar SmithWaterman_non_avx is selected by the
#                      reference's own #ifdef, which needs an x86 <immintrin.h>, so the build is skipped there.
set -euo pipefail
#
#   build_ref.sh --where   prints the checkout's location (nothing where there is none) and builds nothing
REF="${DCNS_REFERENCE:-/root/reference}"
if [ "${1:-}" = "--where" ]; then
  if [ -d "$REF/impl" ]; then echo "$REF"; fi
  exit 0
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/impl" ]; then echo "build_ref: reference checkout not found at $REF; skipped"; exit 0; fi
case "$(uname -m)" in x86_64) ;; *) echo "build_ref: non-x86 host; skipped"; exit 0;; esac
mkdir -p "$OUT"
SRCS="impl/sequenceAlignment3.cpp impl/findSimilarFragmentsForPairedSequence4.cpp impl/slidingWindowAlignment.cpp
      impl/SequenceCharToUInt8.cpp model/Seed.cpp model/Matrix.cpp model/Score.cpp model/PairedSimilarFragment.cpp"
OBJS=""
for s in $SRCS; do
  o="$OUT/$(echo "$s" | tr '/' '_').o"
  g++ -O3 -funroll-all-loops -mavx2 -std=gnu++14 -include cstdint -fPIC -w -I"$REF" -c "$REF/$s" -o "$o" &
  OBJS="$OBJS $o"
done
g++ -O2 -mavx2 -std=gnu++14 -include cstdint -fPIC -w -I"$REF" -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" &
wait
g++ -shared -o "$OUT/libdcns_ref.so" $OBJS "$OUT/ref_harness.o"
echo "build_ref: $OUT/libdcns_ref.so"

# The same reference objects with the dense traceback matrix (model/Matrix.cpp) replaced by oracle/lazy_matrix.cpp,
# which keeps its get/set/reset semantics but stores only the touched cells: pairs of 50-200 kb, whose dense
# (L1+1)(L2+1)-byte matrix does not fit in memory, then run through the unmodified alignment code.
g++ -O2 -std=gnu++14 -include cstdint -fPIC -w -I"$REF" -c "$HERE/lazy_matrix.cpp" -o "$OUT/lazy_matrix.o"
LOBJS="$(echo $OBJS | tr ' ' '\n' | grep -v model_Matrix.cpp.o | tr '\n' ' ')"
g++ -shared -o "$OUT/libdcns_ref_lazy.so" $LOBJS "$OUT/lazy_matrix.o" "$OUT/ref_harness.o"
echo "build_ref: $OUT/libdcns_ref_lazy.so"

# The reference's record writer (outputMasking, controlLayer4.cpp) links against most of the command-line program:
# every non-test source of its CMakeLists target except main.cpp, compiled directly.
CLI="controlLayer4.cpp InputParser.cpp impl/fasta.cpp impl/syntenic.cpp model/Node.cpp model/Graph.cpp
     impl/longestPath.cpp impl/gffToCategory.cpp model/CnsMasResult.cpp model/MsaGraph.cpp
     impl/getCnsForMultipleSpecies.cpp model/PairSequenceAlginmentResult.cpp impl/calculateLambda.cpp
     impl/calculateK.cpp impl/permutationLsqLambdaK.cpp impl/maskGenome.cpp impl/getAllTheCdsPositions.cpp
     impl/samFileToSeeds.cpp model/FastaIndexEntry.cpp impl/FastaIndexEntryImpl.cpp impl/FastaWithIndex.cpp
     model/utils.cpp impl/mapCNSToGenome.cpp"
COBJS=""
for s in $CLI; do
  o="$OUT/cli_$(echo "$s" | tr '/' '_').o"
  g++ -O1 -mavx2 -std=gnu++14 -include cstdint -fPIC -w -I"$REF" -c "$REF/$s" -o "$o" &
  COBJS="$COBJS $o"
done
g++ -O1 -std=gnu++14 -include cstdint -fPIC -w -I"$REF" -c "$HERE/ref_cli_harness.cpp" -o "$OUT/ref_cli_harness.o" &
wait
g++ -shared -o "$OUT/libdcns_ref_cli.so" $OBJS $COBJS "$OUT/ref_cli_harness.o" -lpthread
echo "build_ref: $OUT/libdcns_ref_cli.so"
