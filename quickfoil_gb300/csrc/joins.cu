// joins.cu -- semi-joins and the label-aware binding-set extension.
#include "qfg_common.cuh"

using namespace qfg;

extern "C" int qfg_left_semijoin(qfg_ctx* c, const int32_t* const*, int64_t, const int32_t* const*,
                                 int64_t, int32_t, uint64_t*, int64_t*) {
  if (c == nullptr) return QFG_ERR_INVALID;
  return set_error(&c->impl, QFG_ERR_INVALID, "qfg_left_semijoin: not available in this build");
}

extern "C" int qfg_right_semijoin(qfg_ctx* c, const int32_t* const*, int64_t, const int32_t* const*,
                                  int64_t, int32_t, uint64_t*, int64_t*) {
  if (c == nullptr) return QFG_ERR_INVALID;
  return set_error(&c->impl, QFG_ERR_INVALID, "qfg_right_semijoin: not available in this build");
}

extern "C" int qfg_extend_bindings(qfg_ctx* c, const qfg_bindings*, const qfg_literal*, int64_t,
                                   int64_t, qfg_bindings**) {
  if (c == nullptr) return QFG_ERR_INVALID;
  return set_error(&c->impl, QFG_ERR_INVALID, "qfg_extend_bindings: not available in this build");
}
