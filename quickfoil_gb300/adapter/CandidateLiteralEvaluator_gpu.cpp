// CandidateLiteralEvaluator_gpu.cpp -- compiled in place of the reference's
// learner/CandidateLiteralEvaluator.cpp: the same class
// (learner/CandidateLiteralEvaluator.hpp:23-45), its Evaluate body handing the
// call to qfg_evaluate_group.  The learner above it is unchanged.
//
// Contract kept (learner/CandidateLiteralEvaluator.cpp:264-406): one result
// per literal, appended to *results in the iteration order of
// literal_groups and of each group's vector (LiteralSelector::Insert breaks
// ties by that order); results are new'ed here and deleted by the caller
// (learner/QuickFoil.cpp:429-430); counts are the four CandidateLiteralInfo
// fields (learner/CandidateLiteralInfo.hpp:15-26).  A call whose literals
// have no join result at all gives zeros here, where the reference would
// dereference a null chunk (operations/CountAggregator.cpp:112-116).
#include "learner/CandidateLiteralEvaluator.hpp"

#include <cstdint>
#include <vector>

#include "glog/logging.h"
#include "learner/CandidateLiteralInfo.hpp"
#include "qfgpu_adapter.hpp"

namespace quickfoil {

void CandidateLiteralEvaluator::Evaluate(
    int clause_join_key_id,
    const std::unordered_map<const FoilPredicate*, Vector<const FoilLiteral*>>& literal_groups,
    Vector<CandidateLiteralInfo*>* results) {
  const size_t first = results->size();
  std::vector<qfg_literal> lits;
  for (const auto& group : literal_groups) {
    gpu::EnsureRegistered(group.first);
    for (const FoilLiteral* l : group.second) {
      results->emplace_back(new CandidateLiteralInfo(l));
      lits.push_back(gpu::ToQfgLiteral(*l));
    }
  }
  if (lits.empty()) return;
  gpu::DeviceBindings b = gpu::UploadClause(*building_clause_);
  std::vector<int64_t> counts(4 * lits.size());
  CHECK_EQ(qfg_evaluate_group(gpu::Context(), b.get(), clause_join_key_id, (int32_t)lits.size(),
                              lits.data(), counts.data(), QFG_COUNTS_HOST),
           QFG_OK)
      << qfg_ctx_last_error(gpu::Context());
  for (size_t i = 0; i < lits.size(); ++i) {
    CandidateLiteralInfo* r = (*results)[first + i];
    // int64 in the ABI, size_type (int32) in the reference: counts that
    // reach 2^31 overflow the reference itself.
    r->num_covered_positive = static_cast<size_type>(counts[4 * i + 0]);
    r->num_covered_negative = static_cast<size_type>(counts[4 * i + 1]);
    r->num_binding_positive = static_cast<size_type>(counts[4 * i + 2]);
    r->num_binding_negative = static_cast<size_type>(counts[4 * i + 3]);
  }
}

}  // namespace quickfoil
