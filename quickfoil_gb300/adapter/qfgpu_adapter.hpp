// qfgpu_adapter.hpp -- the C++ side of the drop-in: helpers that hand the
// reference learner's objects (FoilPredicate, FoilClause, FoilLiteral,
// TableView) to libqfgpu's C ABI (include/qfgpu.h).  Compiled together with
// the reference's own sources: CandidateLiteralEvaluator_gpu.cpp replaces
// learner/CandidateLiteralEvaluator.cpp, and the coverage helpers below are
// what the one-line replacement bodies of LiteralSelector::
// ComputeCoveredPositives (learner/LiteralSelector.cpp:150-210) and of the
// counting part of QuickFoil::ComputeCoverageOnUncoveredData
// (learner/QuickFoil.cpp:471-573) call.
//
// Errors: every nonzero status of the C ABI becomes a CHECK failure with the
// context's message, the reference's own reaction to an error.
#ifndef QFGPU_ADAPTER_HPP_
#define QFGPU_ADAPTER_HPP_

#include <memory>

#include "qfgpu.h"
#include "schema/FoilClause.hpp"
#include "schema/FoilLiteral.hpp"
#include "schema/FoilPredicate.hpp"
#include "schema/TypeDefs.hpp"
#include "storage/TableView.hpp"

namespace quickfoil {
namespace gpu {

// The process's context on device 0, created on first use with the
// reference-compatible coverage mode (QFG_OPT_COVERAGE_COMPAT), so coverage
// counts equal the reference's own, chunk-relative tables included.
qfg_ctx* Context();

// Registers a predicate's fact table once per run (relations do not change
// during a learn run); later calls return at once.
void EnsureRegistered(const FoilPredicate* predicate);

// A candidate literal as the C ABI describes it: relation = predicate id,
// vars[i] = the clause variable of argument i (-1 unbound), join_pos =
// FoilLiteral::join_key() (schema/FoilLiteral.hpp:133-144).
qfg_literal ToQfgLiteral(const FoilLiteral& literal);

// A clause's binding set on the device (consecutive or split layout,
// schema/FoilClause.hpp:72-109, 152-161); destroyed with the pointer.
struct BindingsDeleter {
  void operator()(qfg_bindings* b) const;
};
using DeviceBindings = std::unique_ptr<qfg_bindings, BindingsDeleter>;
DeviceBindings UploadClause(const FoilClause& clause);

// A host table (the uncovered positives, the original negatives) on the
// device, as a binding set of positives only: its columns are then device
// columns for qfg_coverage.
DeviceBindings UploadTable(const TableView& table);

// LiteralSelector::ComputeCoveredPositives (learner/LiteralSelector.cpp:
// 150-210): the uncovered positives the literal, appended to `clause`,
// covers.
size_type ComputeCoveredPositives(const FoilClause& clause, const FoilLiteral& literal,
                                  const TableView& uncovered_positive);

// The counts of QuickFoil::ComputeCoverageOnUncoveredData (learner/
// QuickFoil.cpp:471-573): covered uncovered positives and covered original
// negatives; covered_positive_flags (may be null) receives one byte per
// uncovered positive, 1 when covered.
void ComputeCoverage(const FoilClause& clause, const FoilLiteral& literal,
                     const TableView& uncovered_positive, const TableView& negative,
                     size_type* num_positives_covered, size_type* num_negatives_covered,
                     unsigned char* covered_positive_flags);

}  // namespace gpu
}  // namespace quickfoil

#endif  // QFGPU_ADAPTER_HPP_
