// testrun.cu -- the test runner of learnt clauses on the device.
//
// QuickFoilTestRunner::RunTest (learner/QuickFoilTestRunner.cpp:128-161)
// applies the learnt clauses one after another to a test table: for each
// clause the test rows are extended by every body literal but the last
// (CreateBindingTable, operations/MultiColumnHashJoin.cpp:26-115), and the
// last literal's coverage removes the test rows it covers from the ones
// still uncovered (ComputeUnCoveredData, QuickFoilTestRunner.cpp:40-126).
// Here the same chain runs on device-resident tables: the extension's own
// match counts give its size, qfg_extend_bindings builds it,
// qfg_coverage and qfg_compact_rows take the covered rows out.  Nothing but
// the counts crosses to the host between clauses.
#include <cstring>
#include <vector>

#include "qfg_common.cuh"

namespace qfg {

namespace {

// Owns a device binding-set handle.
struct BindingsHandle {
  qfg_ctx* c = nullptr;
  qfg_bindings* b = nullptr;
  ~BindingsHandle() {
    if (b != nullptr) qfg_bindings_destroy(c, b);
  }
  void reset(qfg_bindings* nb) {
    if (b != nullptr) qfg_bindings_destroy(c, b);
    b = nb;
  }
};

}  // namespace

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_run_test(qfg_ctx* c, int32_t num_clauses, const int32_t* clause_lengths,
                            const qfg_literal* body_literals, int32_t num_target_columns,
                            const int32_t* const* d_test_columns, int64_t num_rows,
                            int64_t* num_uncovered, int32_t* const* d_uncovered_out) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  const int k = num_target_columns;
  if (num_uncovered == nullptr || num_clauses < 0 || (num_clauses > 0 && clause_lengths == nullptr) ||
      k < 1 || k > QFG_MAX_ARITY || num_rows < 0 || num_rows > INT32_MAX ||
      (num_rows > 0 && d_test_columns == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_run_test: invalid arguments");
  for (int32_t i = 0; i < num_clauses; ++i)
    if (clause_lengths[i] < 1)
      return set_error(ctx, QFG_ERR_INVALID, "qfg_run_test: a clause needs a body literal");
  *num_uncovered = num_rows;
  if (num_rows == 0) return QFG_OK;
  // Uncovered rows, ping-ponged between two device tables.
  DevBuf buf[2];
  for (int s = 0; s < 2; ++s)
    QFG_TRY(buf[s].reserve(ctx, sizeof(int32_t) * (size_t)k * (size_t)std::max<int64_t>(num_rows, 1)));
  std::vector<int32_t*> cols[2];
  for (int s = 0; s < 2; ++s)
    for (int q = 0; q < k; ++q) cols[s].push_back(buf[s].as<int32_t>() + (size_t)q * num_rows);
  int cur = 0;
  for (int q = 0; q < k && num_rows > 0; ++q)
    QFG_CUDA(ctx, cudaMemcpyAsync(cols[0][q], d_test_columns[q], sizeof(int32_t) * num_rows,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  int64_t left = num_rows;
  DevBuf bits;
  QFG_TRY(bits.reserve(ctx, sizeof(uint64_t) * (size_t)std::max<int64_t>((num_rows + 63) / 64, 1)));
  const qfg_literal* lit = body_literals;
  for (int32_t ci = 0; ci < num_clauses && left > 0; lit += clause_lengths[ci], ++ci) {
    // The clause's bindings start as the test rows (all of them: RunTest
    // extends the full test table, not the uncovered rows).
    BindingsHandle bind;
    bind.c = c;
    qfg_bindings* b0 = nullptr;
    QFG_TRY(qfg_bindings_create(c, k, d_test_columns, num_rows, 0, QFG_DEVICE_BORROW, &b0));
    bind.reset(b0);
    bool empty = false;
    for (int32_t li = 0; li + 1 < clause_lengths[ci] && !empty; ++li) {
      int64_t np = 0, nn = 0;
      QFG_TRY(extension_counts(ctx, bind.b, &lit[li], &np, &nn));
      if (np == 0) {
        empty = true;
        break;
      }
      qfg_bindings* nb = nullptr;
      QFG_TRY(qfg_extend_bindings(c, bind.b, &lit[li], np, 0, &nb));
      bind.reset(nb);
    }
    if (empty) continue;  // the clause covers no test row
    int64_t covered[2] = {0, 0};
    QFG_TRY(qfg_coverage(c, bind.b, &lit[clause_lengths[ci] - 1], k,
                         const_cast<const int32_t* const*>(cols[cur].data()), left, nullptr, 0,
                         bits.as<uint64_t>(), covered));
    if (covered[0] == 0) continue;
    int64_t kept = 0;
    QFG_TRY(qfg_compact_rows(c, k, const_cast<const int32_t* const*>(cols[cur].data()), left,
                             bits.as<uint64_t>(), 0, cols[1 - cur].data(), left, &kept));
    cur = 1 - cur;
    left = kept;
  }
  if (d_uncovered_out != nullptr)
    for (int q = 0; q < k && left > 0; ++q)
      QFG_CUDA(ctx, cudaMemcpyAsync(d_uncovered_out[q], cols[cur][q], sizeof(int32_t) * left,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *num_uncovered = left;
  return QFG_OK;
}
