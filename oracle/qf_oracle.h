/*
 * qf_oracle.h -- CPU oracle for the QuickFOIL candidate-literal hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * operator chain (jbalint/quickfoil), used by tests/, by the smoke check and
 * by the CPU-baseline leg of bench.py as the checker.  Nothing in the product
 * library links, loads or calls it; the product path fails loudly when its
 * CUDA library is missing instead of falling back to this code.
 *
 * Parity pinning: the radix partition restatement is checked against the
 * reference's own RadixPartition_test cases (operations/RadixPartition_test.cpp
 * :106-168); the count restatement is checked against fixtures produced by the
 * reference's own CandidateLiteralEvaluator compiled from its sources (see
 * oracle/build_ref.sh and tests/golden/make_golden.py).
 *
 * Every function names the reference file:line it follows.
 */
#ifndef QF_ORACLE_H_
#define QF_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QFO_MAX_ARITY 8

/* storage/PartitionTuple.hpp:20-42: {int32 value; int32 tuple_id} (8 bytes). */
typedef struct {
  int32_t value;
  int32_t tuple_id;
} qfo_partition_tuple;

/* A column store: num_columns int32 columns of num_tuples rows. */
typedef struct {
  int32_t num_columns;
  int64_t num_tuples;
  const int32_t* const* columns;
} qfo_table;

/* A candidate literal (schema/FoilLiteral.hpp): vars[i] >= 0 is the clause
 * variable bound at argument i (a binding-set column), -1 is unbound.
 * join_pos is FoilLiteral::join_key() (schema/FoilLiteral.hpp:133-144). */
typedef struct {
  int32_t relation;
  int32_t num_args;
  int32_t join_pos;
  int32_t vars[QFO_MAX_ARITY];
} qfo_literal;

/* operations/RadixPartition.cpp:56-155.  Partition id of v is
 * ((uint32_t)v) & (2^bits - 1) (utility/Hash.hpp:18-23, identity hash).
 * Output tuples are grouped by partition and keep input order inside a
 * partition.  offsets[p] .. offsets[p+1] delimit partition p
 * (2^bits + 1 entries). */
void qfo_radix_partition(const int32_t* values, int64_t n, int bits,
                         qfo_partition_tuple* out, int64_t* offsets);

/* storage/FoilHashTable.cpp:34-49: number of buckets = next power of two. */
int32_t qfo_num_buckets(int32_t n);

/* operations/BuildHashTable.cpp:54-93 for one partition of n > 0 tuples:
 * buckets[next_pow2(n)] (1-based chain heads, 0 = empty) and next[n].
 * Returns the FoilHashTable mask ((num_buckets - 1) << bits). */
uint32_t qfo_build_partition_hash_table(const qfo_partition_tuple* part, int32_t n,
                                        int bits, int32_t* buckets, int32_t* next);

/* utility/Hash.hpp:25-55: HashCombine chain over num_keys int32 keys of row
 * tid. */
uint32_t qfo_hash_keys(const int32_t* const* keys, int num_keys, int64_t tid);

/* operations/BuildHashTable.cpp:97-125: whole-table multi-key chained table
 * (radix bits 0).  buckets has next_pow2(n) entries, next has n. */
uint32_t qfo_build_table_hash_table(const int32_t* const* keys, int num_keys, int64_t n,
                                    int32_t* buckets, int32_t* next);

/* BuildHashTableAfterSemiJoin (operations/BuildHashTable.cpp:127-189,
 * 212-236) over the chunks a semi-join yields.  keys are the semi-join's
 * projected columns (num_rows rows); bits (64-bit little-endian blocks)
 * marks the rows that passed.  Chunk c covers rows [c*chunk_rows,
 * min((c+1)*chunk_rows, num_rows)) -- LeftSemiJoin::Next cuts its probe side
 * into FLAGS_semijoin_chunck_size rows and offsets the output columns by
 * the chunk start (operations/LeftSemiJoin.hpp:55-83); chunk_rows <= 0 or
 * >= num_rows is one chunk (RightSemiJoin::Next, operations/
 * RightSemiJoin.hpp:44-82).  Each chunk's set positions are visited in
 * increasing order (BitVectorIterator) and are chunk-relative: the id
 * inserted is the position within the chunk and keys are read at the
 * chunk's rows, also for the positions already in a chain
 * (InsertIfNotPresent, :127-148: inserted at the head of its bucket unless
 * the chain reaches a position with equal keys).  A chain position that
 * lies past the end of a short last chunk (inserted by an earlier chunk)
 * compares unequal; the reference reads past the end of its columns there.
 * The table is
 * FoilHashTable(num_build_tuples, 0): buckets[next_pow2(num_build_tuples)],
 * next[num_build_tuples]; next entries of positions never inserted are 0
 * here (the reference leaves them uninitialised).  num_build_tuples must
 * exceed every chunk-relative position.  Returns the mask. */
uint32_t qfo_build_hash_table_after_semijoin(const int32_t* const* keys, int num_keys,
                                             int64_t num_rows, const uint64_t* bits,
                                             int64_t chunk_rows, int32_t num_build_tuples,
                                             int32_t* buckets, int32_t* next);

/* Relation-partition cache, the analogue of TableView::partitions_
 * (storage/TableView.hpp:62-80): a relation column is partitioned once and
 * reused by every later evaluation (learner/CandidateLiteralEvaluator.cpp:296-299). */
typedef struct qfo_relcache qfo_relcache;
qfo_relcache* qfo_relcache_create(void);
void qfo_relcache_destroy(qfo_relcache* cache);

/* CandidateLiteralEvaluator::Evaluate (learner/CandidateLiteralEvaluator.cpp:
 * 264-406) over one binding set whose first num_positive rows are positive
 * (consecutive layout, :316-343).  For each literal writes four counts to
 * counts[4*i + 0..3] in CandidateLiteralInfo field order
 * (learner/CandidateLiteralInfo.hpp:15-26): num_covered_positive,
 * num_covered_negative, num_binding_positive, num_binding_negative.
 * bits is FLAGS_num_radix_bits; nthreads > 1 evaluates (literal, partition)
 * pairs on that many POSIX threads (the reference is single threaded; the
 * counts do not depend on the thread count).
 * Returns 0 on success, nonzero on an invalid literal. */
int qfo_evaluate(qfo_relcache* cache, const qfo_table* relations, int num_relations,
                 const qfo_table* bindings, int64_t num_positive,
                 const qfo_literal* literals, int num_literals, int bits, int nthreads,
                 int64_t* counts);

/* LeftSemiJoin<k>::DoSemiJoin (operations/LeftSemiJoin.hpp:55-141): one bit
 * per probe row, set when some build row matches on all k keys.  Bits are
 * packed little-endian into 64-bit blocks (utility/BitVector.hpp:25-26).
 * Returns the number of set bits. */
int64_t qfo_left_semijoin(const int32_t* const* probe_keys, int64_t num_probe,
                          const int32_t* const* build_keys, int64_t num_build, int num_keys,
                          uint64_t* out_bits);

/* RightSemiJoin<k>::Next (operations/RightSemiJoin.hpp:44-82): one bit per
 * build row, set when some probe row matches.  Returns the set-bit count. */
int64_t qfo_right_semijoin(const int32_t* const* probe_keys, int64_t num_probe,
                           const int32_t* const* build_keys, int64_t num_build, int num_keys,
                           uint64_t* out_bits);

/* CreateLabelAwareBindingTables (operations/MultiColumnHashJoin.cpp:117-256)
 * for a consecutive binding set.  Output columns: the binding columns then
 * one column per unbound literal argument, positives first.  Rows are
 * produced in the reference's order for the side it would build on.
 * out_columns[c] must hold num_out_positive + num_out_negative rows; the
 * caller takes those counts from the literal's binding counts.  Returns 0,
 * or nonzero when the produced row counts differ from the given ones. */
int qfo_extend_bindings(const qfo_table* bindings, int64_t num_positive,
                        const qfo_table* relation, const qfo_literal* literal,
                        int64_t num_out_positive, int64_t num_out_negative,
                        int32_t* const* out_columns);

/* QuickFoil::ComputeCoverageOnUncoveredData (learner/QuickFoil.cpp:471-573):
 * per label side, the binding rows that pass the left semi-join with the
 * relation on the literal's bound arguments (:494-522) project onto the
 * first num_target_columns binding columns (:504-509); an example is covered
 * when a projection equals it on all of them (:523-541 positives against
 * uncovered_positive, :544-572 negatives against `negative`, which may be
 * NULL).  Restated as set membership, the reference's result wherever its
 * projection table holds whole-table row ids (a label side of at most 32768
 * rows, or one smaller than the relation; operations/BuildHashTable.cpp:
 * 152-189).  positive_bits (may be NULL) receives a bit per uncovered
 * positive (ceil(n/64) blocks).  num_covered[0..1]: covered positives,
 * covered negatives.  Returns 0, or nonzero for an invalid literal. */
int qfo_coverage(const qfo_table* bindings, int64_t num_positive, const qfo_table* relation,
                 const qfo_literal* literal, int num_target_columns,
                 const qfo_table* uncovered_positive, const qfo_table* negative,
                 uint64_t* positive_bits, int64_t* num_covered);

/* ComputeCoverageOnUncoveredData as the reference runs it (the engine's
 * QFG_OPT_COVERAGE_COMPAT): per label side, the bit vector of the side's
 * rows against the relation (its first semi-join), the table
 * BuildHashTableAfterSemiJoin builds from it with chunk-relative positions
 * (32768-row chunks when the side is not smaller than the relation,
 * operations/SemiJoinFactory.cpp:45-82), and the examples probed through
 * that table against the side's rows.  The positive side reads past its end
 * into the negative rows (a view of the consecutive binding columns); past
 * the negative side's end a position compares unequal (the reference reads
 * past its columns).  Same arguments and results as qfo_coverage. */
int qfo_coverage_compat(const qfo_table* bindings, int64_t num_positive, const qfo_table* relation,
                        const qfo_literal* literal, int num_target_columns,
                        const qfo_table* uncovered_positive, const qfo_table* negative,
                        uint64_t* positive_bits, int64_t* num_covered);

/* The compaction of learner/QuickFoil.cpp:655-679 (bit vector flipped, then
 * AttributeReference::EvaluateWithFilter per column): rows whose bit is clear
 * (keep_set 0) or set (keep_set 1), in order, into out[c].  Returns the kept
 * row count. */
int64_t qfo_compact_rows(int num_columns, const int32_t* const* columns, int64_t n,
                         const uint64_t* bits, int keep_set, int32_t* const* out);

/* LoadData (main/main.cpp:49-109) on a text buffer: lines end at '\n'
 * (std::getline); an empty line or one starting with '#' is skipped; fields
 * split at every '|' (boost::split, empty fields kept) must number
 * num_args; every argument not skipped is converted as std::stoi does
 * (FromString<kInt32>, types/FromString.hpp:23-30): leading white space, an
 * optional sign, at least one digit, the value within int32, anything after
 * the digits ignored.  Kept columns go to out[c] (capacity rows each).
 * Returns 0; 1 when capacity is too small (num_rows still set); or, for the
 * first bad line (its 1-based number in *error_line): 2 a field count that
 * differs, 3 a field without digits, 4 a value out of range. */
int qfo_parse_text(const char* text, int64_t n, int num_args, const int32_t* skipped,
                   int32_t* const* out, int64_t capacity, int64_t* num_rows,
                   int64_t* error_line);

#ifdef __cplusplus
}
#endif

#endif /* QF_ORACLE_H_ */
