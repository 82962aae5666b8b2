// Batched persistent launch over many independent SpMMs (placeholder).
#include "internal.h"
using namespace spmm;
struct spmm_batch_plan { int unused; };
extern "C" {
spmm_status spmm_batch_plan_create(const spmm_problem* problems, int count, const spmm_config* cfg,
                                   spmm_batch_plan** plan_out) {
  (void)problems; (void)count; (void)cfg; (void)plan_out;
  return fail(SPMM_ERR_UNSUPPORTED, "batched launch not built yet");
}
spmm_status spmm_batch_run(const spmm_batch_plan* plan, void* stream) {
  (void)plan; (void)stream;
  return fail(SPMM_ERR_UNSUPPORTED, "batched launch not built yet");
}
spmm_status spmm_batch_plan_destroy(spmm_batch_plan* plan) { delete plan; return SPMM_OK; }
}
