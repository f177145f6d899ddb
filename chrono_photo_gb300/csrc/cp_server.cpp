// cp_server.cpp — continuous-batching compositing server (placeholder until the serving
// loop lands: every entry point reports CP_ERR_STATE).
#include "../../include/chrono_gpu.h"

extern "C" {
int cp_server_create(cp_ctx*, uint64_t, int32_t, cp_server** out) {
  if (out) *out = nullptr;
  return CP_ERR_STATE;
}
int cp_server_submit(cp_server*, const cp_job*, uint64_t*) { return CP_ERR_STATE; }
int cp_server_wait(cp_server*, uint64_t, int32_t, cp_job_result*) { return CP_ERR_STATE; }
int cp_server_destroy(cp_server*) { return CP_ERR_STATE; }
}
