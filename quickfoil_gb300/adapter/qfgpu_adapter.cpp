// qfgpu_adapter.cpp -- see qfgpu_adapter.hpp.
#include "qfgpu_adapter.hpp"

#include <cstdint>
#include <unordered_set>
#include <vector>

#include "glog/logging.h"

namespace quickfoil {
namespace gpu {

qfg_ctx* Context() {
  static qfg_ctx* ctx = [] {
    qfg_ctx* c = nullptr;
    CHECK_EQ(qfg_ctx_create(0, 0, &c), QFG_OK) << "qfg_ctx_create";
    CHECK_EQ(qfg_ctx_set_option(c, QFG_OPT_COVERAGE_COMPAT, 1), QFG_OK);
    return c;
  }();
  return ctx;
}

void EnsureRegistered(const FoilPredicate* predicate) {
  static std::unordered_set<int> registered;
  if (!registered.insert(predicate->id()).second) return;
  const TableView& t = predicate->fact_table();
  std::vector<const int32_t*> cols;
  for (int c = 0; c < t.num_columns(); ++c) cols.push_back(t.column_at(c)->as_type<int32_t>());
  CHECK_EQ(qfg_relation_register(Context(), predicate->id(), (int32_t)cols.size(), cols.data(),
                                 (int64_t)t.num_tuples(), QFG_HOST),
           QFG_OK)
      << qfg_ctx_last_error(Context());
}

qfg_literal ToQfgLiteral(const FoilLiteral& literal) {
  qfg_literal d;
  d.relation_id = literal.predicate()->id();
  d.num_args = literal.num_variables();
  d.join_pos = literal.join_key();
  for (int i = 0; i < QFG_MAX_ARITY; ++i)
    d.vars[i] = i < literal.num_variables() && literal.variable_at(i).IsBound()
                    ? literal.variable_at(i).variable_id()
                    : -1;
  return d;
}

void BindingsDeleter::operator()(qfg_bindings* b) const {
  if (b != nullptr) qfg_bindings_destroy(Context(), b);
}

DeviceBindings UploadClause(const FoilClause& clause) {
  std::vector<const int32_t*> pos, neg;
  qfg_bindings* b = nullptr;
  if (clause.IsBindingDataConseuctive()) {
    for (const ConstBufferPtr& blk : clause.integral_blocks()) pos.push_back(blk->as_type<int32_t>());
    CHECK_EQ(qfg_bindings_create(Context(), (int32_t)pos.size(), pos.data(),
                                 clause.GetNumPositiveBindings(), clause.GetNumNegativeBindings(),
                                 QFG_HOST, &b),
             QFG_OK)
        << qfg_ctx_last_error(Context());
  } else {
    for (const ConstBufferPtr& blk : clause.positive_blocks()) pos.push_back(blk->as_type<int32_t>());
    for (const ConstBufferPtr& blk : clause.negative_blocks()) neg.push_back(blk->as_type<int32_t>());
    CHECK_EQ(qfg_bindings_create_split(Context(), (int32_t)pos.size(), pos.data(),
                                       clause.GetNumPositiveBindings(), neg.data(),
                                       clause.GetNumNegativeBindings(), QFG_HOST, &b),
             QFG_OK)
        << qfg_ctx_last_error(Context());
  }
  return DeviceBindings(b);
}

DeviceBindings UploadTable(const TableView& table) {
  std::vector<const int32_t*> cols;
  for (int c = 0; c < table.num_columns(); ++c) cols.push_back(table.column_at(c)->as_type<int32_t>());
  qfg_bindings* b = nullptr;
  CHECK_EQ(qfg_bindings_create(Context(), (int32_t)cols.size(), cols.data(),
                               (int64_t)table.num_tuples(), 0, QFG_HOST, &b),
           QFG_OK)
      << qfg_ctx_last_error(Context());
  return DeviceBindings(b);
}

namespace {

std::vector<const int32_t*> DeviceColumns(const qfg_bindings* b, int k) {
  std::vector<const int32_t*> cols(k, nullptr);
  for (int c = 0; c < k; ++c) CHECK_EQ(qfg_bindings_column(b, c, &cols[c]), QFG_OK);
  return cols;
}

}  // namespace

size_type ComputeCoveredPositives(const FoilClause& clause, const FoilLiteral& literal,
                                  const TableView& uncovered_positive) {
  EnsureRegistered(literal.predicate());
  const int k = clause.head_literal().num_variables();
  DeviceBindings b = UploadClause(clause);
  DeviceBindings u = UploadTable(uncovered_positive);
  const std::vector<const int32_t*> ucols = DeviceColumns(u.get(), k);
  const qfg_literal lit = ToQfgLiteral(literal);
  int64_t covered[2] = {0, 0};
  CHECK_EQ(qfg_coverage(Context(), b.get(), &lit, k, ucols.data(),
                        (int64_t)uncovered_positive.num_tuples(), nullptr, 0, nullptr, covered),
           QFG_OK)
      << qfg_ctx_last_error(Context());
  return static_cast<size_type>(covered[0]);
}

void ComputeCoverage(const FoilClause& clause, const FoilLiteral& literal,
                     const TableView& uncovered_positive, const TableView& negative,
                     size_type* num_positives_covered, size_type* num_negatives_covered,
                     unsigned char* covered_positive_flags) {
  EnsureRegistered(literal.predicate());
  const int k = clause.head_literal().num_variables();
  DeviceBindings b = UploadClause(clause);
  DeviceBindings u = UploadTable(uncovered_positive);
  DeviceBindings n = UploadTable(negative);
  const std::vector<const int32_t*> ucols = DeviceColumns(u.get(), k);
  const std::vector<const int32_t*> ncols = DeviceColumns(n.get(), k);
  const qfg_literal lit = ToQfgLiteral(literal);
  const int64_t nu = (int64_t)uncovered_positive.num_tuples();
  // Device bits for the uncovered positives: kept in a binding set's column
  // storage so that the adapter needs no CUDA headers of its own.
  const int64_t words = 2 * ((nu + 63) / 64);
  std::vector<int32_t> zeros((size_t)std::max<int64_t>(words, 1), 0);
  const int32_t* zcol = zeros.data();
  qfg_bindings* bits_holder = nullptr;
  CHECK_EQ(qfg_bindings_create(Context(), 1, &zcol, std::max<int64_t>(words, 1), 0, QFG_HOST,
                               &bits_holder),
           QFG_OK);
  DeviceBindings bits_owner(bits_holder);
  const int32_t* dbits = nullptr;
  CHECK_EQ(qfg_bindings_column(bits_owner.get(), 0, &dbits), QFG_OK);
  int64_t covered[2] = {0, 0};
  CHECK_EQ(qfg_coverage(Context(), b.get(), &lit, k, ucols.data(), nu, ncols.data(),
                        (int64_t)negative.num_tuples(),
                        reinterpret_cast<uint64_t*>(const_cast<int32_t*>(dbits)), covered),
           QFG_OK)
      << qfg_ctx_last_error(Context());
  *num_positives_covered = static_cast<size_type>(covered[0]);
  *num_negatives_covered = static_cast<size_type>(covered[1]);
  if (covered_positive_flags != nullptr && nu > 0) {
    std::vector<int32_t> host((size_t)words);
    int32_t* hcol = host.data();
    CHECK_EQ(qfg_bindings_download(Context(), bits_owner.get(), &hcol), QFG_OK);
    for (int64_t i = 0; i < nu; ++i)
      covered_positive_flags[i] = (unsigned char)(((uint32_t)host[i >> 5] >> (i & 31)) & 1u);
  }
}

}  // namespace gpu
}  // namespace quickfoil
