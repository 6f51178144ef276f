// ref_driver.cpp -- TEST INFRASTRUCTURE: a C entry layer around the
// reference's own sources (jbalint/quickfoil, compiled unmodified against
// oracle/shims by oracle/build_ref.sh) so that tests can produce golden
// outputs from the real reference code.  Nothing in the product links it.
//
// qfref_evaluate  builds FoilPredicates and a consecutive binding clause from
//                 flat int32 columns and runs CandidateLiteralEvaluator::
//                 Evaluate once per clause join variable, exactly as
//                 QuickFoil::EvaluateAllCandidateLiterals does
//                 (learner/QuickFoil.cpp:418-440).
// qfref_learn     runs QuickFoil::Learn (learner/QuickFoil.cpp:171-359) and,
//                 through link-time wrappers of Evaluate and
//                 CreateLabelAwareBindingTables, writes every call's inputs
//                 and outputs to a trace file.
// qfref_learn_test runs the learner, then QuickFoilTestRunner::RunTest
//                 (learner/QuickFoilTestRunner.cpp:128-161) on test tables.
// qfref_coverage  runs QuickFoil::ComputeCoverageOnUncoveredData
//                 (learner/QuickFoil.cpp:471-573) on a given building clause
//                 (binding set) and uncovered positives: the covered counts
//                 and which uncovered positives are covered.  The method is
//                 private; only this driver's view of the class opens it.
// qfref_learn_compact runs the learner like qfref_learn but writes a compact
//                 trace for knowledge bases of millions of rows: column
//                 checksums in place of columns, and every coverage step
//                 (SelectAndCreateSemiJoin, then the probe of examples
//                 through the after-semijoin table) with its result, seen
//                 through link-time wrappers of the semi-join factory and of
//                 BuildHashTableAfterSemiJoin; it also times the reference
//                 inside each kind of call.
// qfref_build_after_semijoin feeds given chunks (projected columns and a
//                 bit vector, cut into chunk_rows-row chunks as LeftSemiJoin
//                 cuts its probe side) through a stand-in SemiJoin into the
//                 reference's BuildHashTableAfterSemiJoin
//                 (operations/BuildHashTable.cpp:212-236) and returns the
//                 table it builds.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "learner/CandidateLiteralEvaluator.hpp"
#include "learner/CandidateLiteralInfo.hpp"
#include "learner/LiteralSelector.hpp"
#include "learner/QuickFoilState.hpp"
#include "learner/QuickFoilTestRunner.hpp"
#include <chrono>

#include "operations/BuildHashTable.hpp"
#include "operations/SemiJoin.hpp"
#include "operations/SemiJoinFactory.hpp"
#include "storage/TableView.hpp"
#include "storage/FoilHashTable.hpp"
#define private public
#include "learner/QuickFoil.hpp"
#undef private
#include "memory/Buffer.hpp"
#include "operations/MultiColumnHashJoin.hpp"
#include "schema/FoilClause.hpp"
#include "schema/FoilLiteral.hpp"
#include "schema/FoilPredicate.hpp"
#include "schema/FoilVariable.hpp"
#include "utility/Vector.hpp"

#include "gflags/gflags.h"
#include "wrap_names.h"  // generated by oracle/build_ref.sh from the compiled objects

namespace quickfoil {
DECLARE_int32(num_radix_bits);
DECLARE_int32(maximum_clause_length);
}  // namespace quickfoil

using namespace quickfoil;

typedef std::unordered_map<const FoilPredicate*, Vector<const FoilLiteral*>> LiteralGroups;

// The reference's symbols, reached through the linker's --wrap.
void qfref_real_evaluate(CandidateLiteralEvaluator* self, int clause_join_key_id,
                         const LiteralGroups& groups, Vector<CandidateLiteralInfo*>* results)
    asm("__real_" QFREF_EVALUATE);
void qfref_real_extend(const FoilClauseConstSharedPtr& clause, const FoilLiteral& literal,
                       const size_type num_pos, const size_type num_neg,
                       Vector<ConstBufferPtr>* new_table)
    asm("__real_" QFREF_EXTEND);
SemiJoin* qfref_real_select(const TableView& output_table, const TableView& other_table,
                            std::unique_ptr<FoilHashTable>* output_hash_table,
                            std::unique_ptr<FoilHashTable>* other_hash_table,
                            const Vector<AttributeReference>& output_join_keys,
                            const Vector<AttributeReference>& other_join_keys,
                            const Vector<int>& project_column_ids)
    asm("__real_" QFREF_SELECT);
SemiJoin* qfref_real_create(bool left_semijoin, const TableView& probe_table,
                            const TableView& build_table, const FoilHashTable& build_hash_table,
                            const Vector<AttributeReference>& probe_keys,
                            const Vector<AttributeReference>& build_keys,
                            const Vector<int>& project_column_ids)
    asm("__real_" QFREF_CREATE);
FoilHashTable* qfref_real_after(const size_type num_build_tuples, int num_build_keys,
                                SemiJoin* semi_join)
    asm("__real_" QFREF_AFTER);

namespace {

FILE* g_trace = nullptr;
// Compact trace (qfref_learn_compact): checksums instead of columns, and
// the coverage steps.
bool g_compact = false;
// Fact-table column 0 data pointer -> relation index (identifies a
// literal's relation in SelectAndCreateSemiJoin).
std::unordered_map<const void*, int> g_rel_of_column;
// Seconds the reference spent inside each kind of traced call.
double g_sec_evaluate = 0, g_sec_extend = 0, g_sec_coverage = 0;

double Now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Checksum of an int32 column: sum over rows r of ((uint32)v + 0x9e3779b9) *
// (2r + 1), modulo 2^64 (tests/golden computes the same on the device).
uint64_t ColumnChecksum(const int32_t* v, int64_t n) {
  uint64_t s = 0;
  for (int64_t r = 0; r < n; ++r) s += ((uint64_t)(uint32_t)v[r] + 0x9e3779b9ull) * (uint64_t)(2 * r + 1);
  return s;
}

ConstBufferPtr MakeColumn(const int32_t* src, int64_t n) {
  BufferPtr b = std::make_shared<Buffer>(sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1), (size_t)n);
  if (n > 0) memcpy(b->mutable_data(), src, sizeof(int32_t) * (size_t)n);
  return std::make_shared<const ConstBuffer>(b);
}

Vector<ConstBufferPtr> MakeColumns(int ncols, const int32_t* const* cols, int64_t n) {
  Vector<ConstBufferPtr> out;
  for (int c = 0; c < ncols; ++c) out.emplace_back(MakeColumn(cols[c], n));
  return out;
}

void WriteColumn(const char* tag, const int32_t* v, int64_t n) {
  if (g_compact) {
    fprintf(g_trace, "%sCS %llu\n", tag, (unsigned long long)ColumnChecksum(v, n));
    return;
  }
  fprintf(g_trace, "%s", tag);
  for (int64_t i = 0; i < n; ++i) fprintf(g_trace, " %d", v[i]);
  fprintf(g_trace, "\n");
}

// Binding set of a clause as consecutive columns (positives then negatives).
void WriteBindings(const FoilClause& clause) {
  const int64_t P = clause.GetNumPositiveBindings(), N = clause.GetNumNegativeBindings();
  const int ncols = clause.num_variables();
  fprintf(g_trace, "BINDINGS %d %lld %lld\n", ncols, (long long)P, (long long)N);
  for (int c = 0; c < ncols; ++c) {
    std::vector<int32_t> col;
    if (clause.IsBindingDataConseuctive()) {
      const int32_t* v = clause.integral_blocks()[c]->as_type<int32_t>();
      col.assign(v, v + P + N);
    } else {
      const int32_t* p = clause.positive_blocks()[c]->as_type<int32_t>();
      const int32_t* q = clause.negative_blocks()[c]->as_type<int32_t>();
      col.assign(p, p + P);
      col.insert(col.end(), q, q + N);
    }
    WriteColumn("COL", col.data(), (int64_t)col.size());
  }
}

void WriteLiteral(const char* tag, const FoilLiteral& l) {
  fprintf(g_trace, "%s %d %d %d", tag, l.predicate()->id(), l.num_variables(), l.join_key());
  for (int i = 0; i < l.num_variables(); ++i) fprintf(g_trace, " %d", l.variable_at(i).variable_id());
  fprintf(g_trace, "\n");
}

// The reference crashes when no literal of a call has any join-key match
// (operations/CountAggregator.cpp:112-116 dereferences the first, null,
// chunk).  Such a call's counts are all zero, so it is answered directly.
bool CallHasJoinResult(const FoilClause& clause, int join_var, const LiteralGroups& groups) {
  std::unordered_set<int32_t> keys;
  const int64_t total = clause.GetNumTotalBindings();
  if (clause.IsBindingDataConseuctive()) {
    const int32_t* v = clause.integral_blocks()[join_var]->as_type<int32_t>();
    keys.insert(v, v + total);
  } else {
    const int32_t* p = clause.positive_blocks()[join_var]->as_type<int32_t>();
    const int32_t* q = clause.negative_blocks()[join_var]->as_type<int32_t>();
    keys.insert(p, p + clause.GetNumPositiveBindings());
    keys.insert(q, q + clause.GetNumNegativeBindings());
  }
  for (const auto& g : groups) {
    for (const FoilLiteral* l : g.second) {
      const TableView& t = l->predicate()->fact_table();
      const int32_t* col = t.column_at(l->join_key())->as_type<int32_t>();
      for (int64_t i = 0; i < t.num_tuples(); ++i)
        if (keys.count(col[i])) return true;
    }
  }
  return false;
}

// CandidateLiteralEvaluator holds only `const FoilClauseConstSharedPtr&
// building_clause_` (learner/CandidateLiteralEvaluator.hpp:42): one pointer.
const FoilClause& EvaluatorClause(const CandidateLiteralEvaluator* self) {
  static_assert(sizeof(CandidateLiteralEvaluator) == sizeof(void*), "evaluator layout");
  const FoilClauseConstSharedPtr* p = *reinterpret_cast<const FoilClauseConstSharedPtr* const*>(self);
  return **p;
}

}  // namespace

void qfref_wrap_evaluate(CandidateLiteralEvaluator* self, int clause_join_key_id,
                         const LiteralGroups& groups, Vector<CandidateLiteralInfo*>* results)
    asm("__wrap_" QFREF_EVALUATE);
void qfref_wrap_evaluate(CandidateLiteralEvaluator* self, int clause_join_key_id,
                         const LiteralGroups& groups, Vector<CandidateLiteralInfo*>* results) {
  const FoilClause& clause = EvaluatorClause(self);
  const size_t before = results->size();
  if (CallHasJoinResult(clause, clause_join_key_id, groups)) {
    const double t0 = Now();
    qfref_real_evaluate(self, clause_join_key_id, groups, results);
    g_sec_evaluate += Now() - t0;
  } else {
    for (const auto& g : groups)
      for (const FoilLiteral* l : g.second) results->emplace_back(new CandidateLiteralInfo(l));
  }
  if (g_trace != nullptr) {
    fprintf(g_trace, "EVALUATE %d %zu\n", clause_join_key_id, results->size() - before);
    WriteBindings(clause);
    for (size_t i = before; i < results->size(); ++i) {
      const CandidateLiteralInfo* r = (*results)[i];
      WriteLiteral("LIT", *r->literal);
      fprintf(g_trace, "COUNTS %d %d %d %d\n", r->num_covered_positive, r->num_covered_negative,
              r->num_binding_positive, r->num_binding_negative);
    }
  }
}

void qfref_wrap_extend(const FoilClauseConstSharedPtr& clause, const FoilLiteral& literal,
                       const size_type num_pos, const size_type num_neg,
                       Vector<ConstBufferPtr>* new_table)
    asm("__wrap_" QFREF_EXTEND);
void qfref_wrap_extend(const FoilClauseConstSharedPtr& clause, const FoilLiteral& literal,
                       const size_type num_pos, const size_type num_neg,
                       Vector<ConstBufferPtr>* new_table) {
  const size_t before = new_table->size();
  const double t0 = Now();
  qfref_real_extend(clause, literal, num_pos, num_neg, new_table);
  g_sec_extend += Now() - t0;
  if (g_trace != nullptr) {
    fprintf(g_trace, "EXTEND %d %d\n", num_pos, num_neg);
    WriteBindings(*clause);
    WriteLiteral("LIT", literal);
    for (size_t c = before; c < new_table->size(); ++c)
      WriteColumn("OUT", (*new_table)[c]->as_type<int32_t>(), num_pos + num_neg);
  }
}

namespace {

// Forwards a semi-join's chunks and, once it is exhausted, writes the
// probe's result to the trace: the set-bit count and two sums over the set
// positions e (sum of e + 1 and of (e + 1)^2, modulo 2^64).
class RecordingSemiJoin : public SemiJoin {
 public:
  RecordingSemiJoin(const TableView& empty, const FoilHashTable& table, SemiJoin* inner,
                    int64_t probe_rows, int64_t build_rows)
      : SemiJoin(empty, empty, table, Vector<AttributeReference>(), Vector<AttributeReference>(),
                 Vector<int>()),
        inner_(inner), probe_rows_(probe_rows), build_rows_(build_rows) {}

  SemiJoinChunk* Next() override {
    const double t0 = Now();
    SemiJoinChunk* c = inner_->Next();
    g_sec_coverage += Now() - t0;
    if (c != nullptr) {
      ones_ += (int64_t)c->num_ones;
      for (size_t i = 0; i < c->semi_bitvector.size(); ++i) {
        if (!c->semi_bitvector.test(i)) continue;
        const uint64_t e = (uint64_t)(seen_ + (int64_t)i) + 1;
        s1_ += e;
        s2_ += e * e;
      }
      seen_ += (int64_t)c->semi_bitvector.size();
    } else if (!done_) {
      done_ = true;
      if (g_trace != nullptr)
        fprintf(g_trace, "PROBE %lld %lld %lld %llu %llu\n", (long long)probe_rows_,
                (long long)build_rows_, (long long)ones_, (unsigned long long)s1_,
                (unsigned long long)s2_);
    }
    return c;
  }

 private:
  std::unique_ptr<SemiJoin> inner_;
  int64_t probe_rows_, build_rows_;
  int64_t ones_ = 0, seen_ = 0;
  uint64_t s1_ = 0, s2_ = 0;
  bool done_ = false;
};

TableView& EmptyTable() {
  static TableView* t = new TableView(Vector<ConstBufferPtr>());
  return *t;
}
FoilHashTable& DummyTable() {
  static FoilHashTable* t = new FoilHashTable(1, 0);
  return *t;
}

void WriteTableChecksums(const char* tag, const TableView& t) {
  fprintf(g_trace, "%s %lld", tag, (long long)t.num_tuples());
  for (int c = 0; c < t.num_columns(); ++c)
    fprintf(g_trace, " %llu", (unsigned long long)ColumnChecksum(
                                  t.column_at(c)->as_type<int32_t>(), (int64_t)t.num_tuples()));
  fprintf(g_trace, "\n");
}

}  // namespace

SemiJoin* qfref_wrap_select(const TableView& output_table, const TableView& other_table,
                            std::unique_ptr<FoilHashTable>* output_hash_table,
                            std::unique_ptr<FoilHashTable>* other_hash_table,
                            const Vector<AttributeReference>& output_join_keys,
                            const Vector<AttributeReference>& other_join_keys,
                            const Vector<int>& project_column_ids)
    asm("__wrap_" QFREF_SELECT);
SemiJoin* qfref_wrap_select(const TableView& output_table, const TableView& other_table,
                            std::unique_ptr<FoilHashTable>* output_hash_table,
                            std::unique_ptr<FoilHashTable>* other_hash_table,
                            const Vector<AttributeReference>& output_join_keys,
                            const Vector<AttributeReference>& other_join_keys,
                            const Vector<int>& project_column_ids) {
  if (g_trace != nullptr && g_compact) {
    auto it = g_rel_of_column.find(other_table.column_at(0)->data());
    // SELJ <relation> <bound argument count> (binding column, relation
    // argument)... then the label side's row count and column checksums.
    fprintf(g_trace, "SELJ %d %d", it == g_rel_of_column.end() ? -1 : it->second,
            (int)output_join_keys.size());
    for (size_t i = 0; i < output_join_keys.size(); ++i)
      fprintf(g_trace, " %d %d", output_join_keys[i].column_id(), other_join_keys[i].column_id());
    fprintf(g_trace, "\n");
    WriteTableChecksums("SIDE", output_table);
  }
  const double t0 = Now();
  SemiJoin* sj = qfref_real_select(output_table, other_table, output_hash_table, other_hash_table,
                                   output_join_keys, other_join_keys, project_column_ids);
  g_sec_coverage += Now() - t0;
  return sj;
}

FoilHashTable* qfref_wrap_after(const size_type num_build_tuples, int num_build_keys,
                                SemiJoin* semi_join)
    asm("__wrap_" QFREF_AFTER);
FoilHashTable* qfref_wrap_after(const size_type num_build_tuples, int num_build_keys,
                                SemiJoin* semi_join) {
  const double t0 = Now();
  FoilHashTable* t = qfref_real_after(num_build_tuples, num_build_keys, semi_join);
  g_sec_coverage += Now() - t0;
  return t;
}

SemiJoin* qfref_wrap_create(bool left_semijoin, const TableView& probe_table,
                            const TableView& build_table, const FoilHashTable& build_hash_table,
                            const Vector<AttributeReference>& probe_keys,
                            const Vector<AttributeReference>& build_keys,
                            const Vector<int>& project_column_ids)
    asm("__wrap_" QFREF_CREATE);
SemiJoin* qfref_wrap_create(bool left_semijoin, const TableView& probe_table,
                            const TableView& build_table, const FoilHashTable& build_hash_table,
                            const Vector<AttributeReference>& probe_keys,
                            const Vector<AttributeReference>& build_keys,
                            const Vector<int>& project_column_ids) {
  const double t0 = Now();
  SemiJoin* sj = qfref_real_create(left_semijoin, probe_table, build_table, build_hash_table,
                                   probe_keys, build_keys, project_column_ids);
  g_sec_coverage += Now() - t0;
  if (g_trace == nullptr || !g_compact) return sj;
  // The examples probed (uncovered positives or original negatives).
  WriteTableChecksums("EXAMPLES", probe_table);
  return new RecordingSemiJoin(EmptyTable(), DummyTable(), sj, (int64_t)probe_table.num_tuples(),
                               (int64_t)build_table.num_tuples());
}

namespace {

// A SemiJoin that yields fixed chunks: rows [c0, c0 + chunk_rows) of the
// given columns (offset by the chunk start, as LeftSemiJoin::Next offsets its
// output columns) with their bits.  Its base is built on empty tables and no
// keys, so the base constructor reads nothing.
class ChunkFeed : public SemiJoin {
 public:
  ChunkFeed(const TableView& empty, const FoilHashTable& table, int nkeys,
            const int32_t* const* keys, int64_t n, const uint64_t* bits, int64_t chunk_rows)
      : SemiJoin(empty, empty, table, Vector<AttributeReference>(), Vector<AttributeReference>(),
                 Vector<int>()),
        nkeys_(nkeys), keys_(keys), n_(n), bits_(bits),
        chunk_(chunk_rows <= 0 || chunk_rows > n ? n : chunk_rows) {}

  SemiJoinChunk* Next() override {
    if (c0_ >= n_) return nullptr;
    const int64_t len = std::min<int64_t>(chunk_, n_ - c0_);
    Vector<const cpp_type*> cols;
    for (int k = 0; k < nkeys_; ++k) cols.emplace_back(keys_[k] + c0_);
    BitVector bv((size_t)len);
    for (int64_t i = 0; i < len; ++i) {
      const int64_t r = c0_ + i;
      if ((bits_[r >> 6] >> (r & 63)) & 1u) bv.set((size_t)i);
    }
    c0_ += chunk_;
    return new SemiJoinChunk(std::move(cols), std::move(bv));
  }

 private:
  int nkeys_;
  const int32_t* const* keys_;
  int64_t n_;
  const uint64_t* bits_;
  int64_t chunk_;
  int64_t c0_ = 0;
};

}  // namespace

extern "C" {

// The reference's BuildHashTableAfterSemiJoin over the chunks of `keys`
// (nkeys columns of n rows) and `bits`; buckets receives next_pow2(
// num_build_tuples) heads, next[] num_build_tuples links (entries of
// positions the reference never wrote are set to 0), *mask the mask.
int qfref_build_after_semijoin(int nkeys, const int32_t* const* keys, int64_t n,
                               const uint64_t* bits, int64_t chunk_rows,
                               int32_t num_build_tuples, int32_t* buckets, int32_t* next,
                               uint32_t* mask) {
  if (n <= 0 || num_build_tuples <= 0) return 1;
  TableView empty{Vector<ConstBufferPtr>()};
  FoilHashTable dummy(1, 0);
  // The reference leaves next[] of never-inserted positions uninitialised:
  // they are recognised as positions that no chain reaches.
  std::unique_ptr<FoilHashTable> t(BuildHashTableAfterSemiJoin(
      (size_type)num_build_tuples, nkeys,
      new ChunkFeed(empty, dummy, nkeys, keys, n, bits, chunk_rows)));
  int32_t nb = num_build_tuples - 1;
  nb |= nb >> 1; nb |= nb >> 2; nb |= nb >> 4; nb |= nb >> 8; nb |= nb >> 16;
  nb += 1;
  memcpy(buckets, t->buckets(), sizeof(int32_t) * (size_t)nb);
  std::vector<char> reached((size_t)num_build_tuples, 0);
  for (int32_t b = 0; b < nb; ++b)
    for (int32_t pos = buckets[b] - 1; pos >= 0 && !reached[pos]; pos = t->next()[pos] - 1)
      reached[pos] = 1;
  for (int32_t i = 0; i < num_build_tuples; ++i) next[i] = reached[i] ? t->next()[i] : 0;
  *mask = t->mask();
  return 0;
}

// Literal descriptors: lits[k * 10 + 0] = relation index, [1] = number of
// arguments, [2 .. 9] = clause variable per argument (-1 unbound).  All
// arguments share one type, so the join key is the first bound argument.
int qfref_evaluate(int nrel, const int* rel_ncols, const int64_t* rel_ntuples,
                   const int32_t* const* rel_cols, int bind_ncols, const int32_t* const* bind_cols,
                   int64_t npos, int64_t nneg, int nlits, const int32_t* lits, int radix_bits,
                   int64_t* counts) {
  FLAGS_num_radix_bits = radix_bits;
  std::vector<std::unique_ptr<FoilPredicate>> preds;
  int off = 0;
  for (int r = 0; r < nrel; ++r) {
    Vector<int> types(rel_ncols[r], 0);
    preds.emplace_back(new FoilPredicate(r, "r" + std::to_string(r), -1, types,
                                         MakeColumns(rel_ncols[r], rel_cols + off, rel_ntuples[r])));
    off += rel_ncols[r];
  }
  Vector<int> head_types(bind_ncols, 0);
  FoilPredicate head_pred(nrel, "head", -1, head_types, MakeColumns(bind_ncols, bind_cols, 0));
  FoilLiteral head(&head_pred);
  for (int c = 0; c < bind_ncols; ++c) head.AddVariable(FoilVariable(c, 0));
  FoilClauseConstSharedPtr clause = FoilClause::Create(
      head, (size_type)npos, (size_type)nneg, MakeColumns(bind_ncols, bind_cols, npos + nneg));

  std::vector<std::unique_ptr<FoilLiteral>> literals;
  for (int k = 0; k < nlits; ++k) {
    const int32_t* d = lits + 10 * k;
    if (d[0] < 0 || d[0] >= nrel || d[1] != rel_ncols[d[0]]) return 1;
    Vector<FoilVariable> vars;
    for (int i = 0; i < d[1]; ++i) vars.emplace_back(d[2 + i] >= 0 ? FoilVariable(d[2 + i], 0) : FoilVariable(0));
    literals.emplace_back(new FoilLiteral(preds[d[0]].get(), vars));
    if (literals.back()->join_key() < 0) return 2;
  }
  memset(counts, 0, sizeof(int64_t) * 4 * (size_t)nlits);
  CandidateLiteralEvaluator evaluator(clause);
  for (int var = 0; var < bind_ncols; ++var) {
    LiteralGroups groups;
    for (auto& l : literals)
      if (l->variable_at(l->join_key()).variable_id() == var) groups[l->predicate()].emplace_back(l.get());
    if (groups.empty()) continue;
    Vector<CandidateLiteralInfo*> results;
    evaluator.Evaluate(var, groups, &results);
    for (CandidateLiteralInfo* r : results) {
      for (int k = 0; k < nlits; ++k) {
        if (literals[k].get() != r->literal) continue;
        counts[4 * k + 0] = r->num_covered_positive;
        counts[4 * k + 1] = r->num_covered_negative;
        counts[4 * k + 2] = r->num_binding_positive;
        counts[4 * k + 3] = r->num_binding_negative;
      }
      delete r;
    }
  }
  return 0;
}

// Runs the reference learner on one target relation (positives first) and
// background relations; writes the learnt clauses (one per line) to
// `clauses` and, when trace_path is given, every Evaluate and
// CreateLabelAwareBindingTables call to that file.
int qfref_learn(int nrel, const int* rel_ncols, const int64_t* rel_ntuples,
                const int32_t* const* rel_cols, int target_ncols, int64_t target_n,
                int64_t target_npos, const int32_t* const* target_cols, int max_clause_length,
                const char* trace_path, char* clauses, int clauses_cap) {
  FLAGS_maximum_clause_length = max_clause_length;
  std::vector<std::unique_ptr<FoilPredicate>> owned;
  Vector<const FoilPredicate*> background;
  int off = 0;
  for (int r = 0; r < nrel; ++r) {
    Vector<int> types(rel_ncols[r], 0);
    owned.emplace_back(new FoilPredicate(r, "r" + std::to_string(r), -1, types,
                                         MakeColumns(rel_ncols[r], rel_cols + off, rel_ntuples[r])));
    background.push_back(owned.back().get());
    off += rel_ncols[r];
  }
  Vector<int> ttypes(target_ncols, 0);
  FoilPredicate target(nrel, "target", -1, ttypes, MakeColumns(target_ncols, target_cols, target_n));
  if (trace_path != nullptr) {
    g_trace = fopen(trace_path, "w");
    if (g_trace == nullptr) return 3;
  }
  std::string out;
  {
    QuickFoil qf((size_type)target_npos, (size_type)(target_n - target_npos), &target, background);
    qf.Learn();
    for (const auto& c : qf.learnt_clauses()) out += c->ToString() + "\n";
  }
  if (g_trace != nullptr) {
    fprintf(g_trace, "CLAUSES\n%sEND\n", out.c_str());
    fclose(g_trace);
    g_trace = nullptr;
  }
  if (clauses != nullptr && clauses_cap > 0) {
    strncpy(clauses, out.c_str(), (size_t)clauses_cap - 1);
    clauses[clauses_cap - 1] = '\0';
  }
  return 0;
}

// qfref_learn with the compact trace (see the top of this file); seconds[0..3]
// receive the reference's time in Learn as a whole, inside Evaluate, inside
// CreateLabelAwareBindingTables and inside the coverage steps.
int qfref_learn_compact(int nrel, const int* rel_ncols, const int64_t* rel_ntuples,
                        const int32_t* const* rel_cols, int target_ncols, int64_t target_n,
                        int64_t target_npos, const int32_t* const* target_cols,
                        int max_clause_length, const char* trace_path, char* clauses,
                        int clauses_cap, double* seconds) {
  FLAGS_maximum_clause_length = max_clause_length;
  std::vector<std::unique_ptr<FoilPredicate>> owned;
  Vector<const FoilPredicate*> background;
  int off = 0;
  g_rel_of_column.clear();
  for (int r = 0; r < nrel; ++r) {
    Vector<int> types(rel_ncols[r], 0);
    owned.emplace_back(new FoilPredicate(r, "r" + std::to_string(r), -1, types,
                                         MakeColumns(rel_ncols[r], rel_cols + off, rel_ntuples[r])));
    background.push_back(owned.back().get());
    g_rel_of_column[owned.back()->fact_table().column_at(0)->data()] = r;
    off += rel_ncols[r];
  }
  Vector<int> ttypes(target_ncols, 0);
  FoilPredicate target(nrel, "target", -1, ttypes, MakeColumns(target_ncols, target_cols, target_n));
  g_trace = fopen(trace_path, "w");
  if (g_trace == nullptr) return 3;
  g_compact = true;
  g_sec_evaluate = g_sec_extend = g_sec_coverage = 0;
  std::string out;
  double learn_s = 0;
  {
    QuickFoil qf((size_type)target_npos, (size_type)(target_n - target_npos), &target, background);
    const double t0 = Now();
    qf.Learn();
    learn_s = Now() - t0;
    for (const auto& c : qf.learnt_clauses()) out += c->ToString() + "\n";
  }
  fprintf(g_trace, "CLAUSES\n%sEND\n", out.c_str());
  fclose(g_trace);
  g_trace = nullptr;
  g_compact = false;
  seconds[0] = learn_s;
  seconds[1] = g_sec_evaluate;
  seconds[2] = g_sec_extend;
  seconds[3] = g_sec_coverage;
  if (clauses != nullptr && clauses_cap > 0) {
    strncpy(clauses, out.c_str(), (size_t)clauses_cap - 1);
    clauses[clauses_cap - 1] = '\0';
  }
  return 0;
}

// Runs the reference learner as qfref_learn does, then its test runner
// (learner/QuickFoilTestRunner.cpp:128-161) on a positive and a negative
// test table (test_ncols = target columns): uncovered[0] / [1] receive the
// test rows no learnt clause covers.
int qfref_learn_test(int nrel, const int* rel_ncols, const int64_t* rel_ntuples,
                     const int32_t* const* rel_cols, int target_ncols, int64_t target_n,
                     int64_t target_npos, const int32_t* const* target_cols,
                     int max_clause_length, int64_t test_npos,
                     const int32_t* const* test_pos_cols, int64_t test_nneg,
                     const int32_t* const* test_neg_cols, char* clauses, int clauses_cap,
                     int64_t* uncovered) {
  FLAGS_maximum_clause_length = max_clause_length;
  std::vector<std::unique_ptr<FoilPredicate>> owned;
  Vector<const FoilPredicate*> background;
  int off = 0;
  for (int r = 0; r < nrel; ++r) {
    Vector<int> types(rel_ncols[r], 0);
    owned.emplace_back(new FoilPredicate(r, "r" + std::to_string(r), -1, types,
                                         MakeColumns(rel_ncols[r], rel_cols + off, rel_ntuples[r])));
    background.push_back(owned.back().get());
    off += rel_ncols[r];
  }
  Vector<int> ttypes(target_ncols, 0);
  FoilPredicate target(nrel, "target", -1, ttypes, MakeColumns(target_ncols, target_cols, target_n));
  QuickFoil qf((size_type)target_npos, (size_type)(target_n - target_npos), &target, background);
  qf.Learn();
  std::string out;
  for (const auto& c : qf.learnt_clauses()) out += c->ToString() + "\n";
  if (clauses != nullptr && clauses_cap > 0) {
    strncpy(clauses, out.c_str(), (size_t)clauses_cap - 1);
    clauses[clauses_cap - 1] = '\0';
  }
  QuickFoilTestRunner runner(&target, qf.learnt_clauses());
  TableView pos(MakeColumns(target_ncols, test_pos_cols, test_npos));
  TableView neg(MakeColumns(target_ncols, test_neg_cols, test_nneg));
  uncovered[0] = (int64_t)runner.RunTest(pos);
  uncovered[1] = (int64_t)runner.RunTest(neg);
  return 0;
}

// The reference's coverage computation for one literal appended to a
// building clause: binding set (bind_npos positives then bind_nneg
// negatives, bind_ncols columns, the first target_ncols of them the target's
// variables), the uncovered positives (unc_n rows of target_ncols columns),
// and the target (positives first; its negatives are the reference's
// original negative data).  Writes covered positive / negative counts and,
// per uncovered positive, 1 when covered.
int qfref_coverage(int nrel, const int* rel_ncols, const int64_t* rel_ntuples,
                   const int32_t* const* rel_cols, int target_ncols, int64_t target_n,
                   int64_t target_npos, const int32_t* const* target_cols, int bind_ncols,
                   int64_t bind_npos, int64_t bind_nneg, const int32_t* const* bind_cols,
                   const int32_t* lit, int64_t unc_n, const int32_t* const* unc_cols,
                   int64_t* counts, uint8_t* covered) {
  std::vector<std::unique_ptr<FoilPredicate>> owned;
  Vector<const FoilPredicate*> background;
  int off = 0;
  for (int r = 0; r < nrel; ++r) {
    Vector<int> types(rel_ncols[r], 0);
    owned.emplace_back(new FoilPredicate(r, "r" + std::to_string(r), -1, types,
                                         MakeColumns(rel_ncols[r], rel_cols + off, rel_ntuples[r])));
    background.push_back(owned.back().get());
    off += rel_ncols[r];
  }
  if (lit[0] < 0 || lit[0] >= nrel || lit[1] != rel_ncols[lit[0]]) return 1;
  Vector<int> ttypes(target_ncols, 0);
  FoilPredicate target(nrel, "target", -1, ttypes, MakeColumns(target_ncols, target_cols, target_n));
  QuickFoil qf((size_type)target_npos, (size_type)(target_n - target_npos), &target, background);
  FoilLiteral head(&target);
  for (int c = 0; c < target_ncols; ++c) head.AddVariable(FoilVariable(c, 0));
  qf.building_state_->building_clause = FoilClause::Create(
      head, (size_type)bind_npos, (size_type)bind_nneg,
      MakeColumns(bind_ncols, bind_cols, bind_npos + bind_nneg));
  Vector<ConstBufferPtr> unc = MakeColumns(target_ncols, unc_cols, unc_n);
  qf.building_state_->uncovered_positive_data = std::make_shared<TableView>(std::move(unc));
  Vector<FoilVariable> vars;
  for (int i = 0; i < lit[1]; ++i) vars.emplace_back(lit[2 + i] >= 0 ? FoilVariable(lit[2 + i], 0) : FoilVariable(0));
  FoilLiteral literal(owned[lit[0]].get(), vars);
  std::unique_ptr<FoilHashTable> table;
  size_type npos = 0, nneg = 0;
  Vector<SemiJoinChunk*> chunks;
  qf.ComputeCoverageOnUncoveredData(literal, &table, &npos, &nneg, &chunks);
  counts[0] = npos;
  counts[1] = nneg;
  memset(covered, 0, (size_t)unc_n);
  const int32_t* base = qf.building_state_->uncovered_positive_data->column_at(0)->as_type<int32_t>();
  for (SemiJoinChunk* c : chunks) {
    const int64_t first = c->output_columns[0] - base;
    for (size_t i = 0; i < c->semi_bitvector.size(); ++i)
      if (c->semi_bitvector.test(i)) covered[first + (int64_t)i] = 1;
    delete c;
  }
  return 0;
}

}  // extern "C"
