// sgb_batch.cu -- replica batches and parallel tempering (ParallelTempering.jl:2-95).
#include <cuda_runtime.h>
#include <string>
#include "sgb_internal.h"

struct sgb_batch {
    std::string err;
};

extern "C" {

static const char* k_unimpl = "replica batches are not available in this build";

int sgb_batch_create(const sgb_desc*, int32_t, const int32_t*, sgb_batch** out) {
    if (out) *out = nullptr;
    return SGB_ERR_STATE;
}
void sgb_batch_destroy(sgb_batch* b) { delete b; }
const char* sgb_batch_last_error(const sgb_batch*) { return k_unimpl; }
int64_t sgb_batch_nsites(const sgb_batch*, int32_t) { return 0; }
int sgb_batch_set_couplings(sgb_batch*, const double*, const double*, const double*, const double*, const sgb_bond*, int32_t) { return SGB_ERR_STATE; }
int sgb_batch_set_state(sgb_batch*, int32_t, const double*) { return SGB_ERR_STATE; }
int sgb_batch_get_state(sgb_batch*, int32_t, double*) { return SGB_ERR_STATE; }
int sgb_batch_set_kT(sgb_batch*, const double*) { return SGB_ERR_STATE; }
int sgb_batch_get_kT(sgb_batch*, double*) { return SGB_ERR_STATE; }
int sgb_batch_langevin(sgb_batch*, double, double, uint64_t, uint64_t, int32_t) { return SGB_ERR_STATE; }
int sgb_batch_energy(sgb_batch*, double*) { return SGB_ERR_STATE; }
int sgb_batch_exchange(sgb_batch*, int32_t, uint64_t, uint64_t, const double*, int64_t*) { return SGB_ERR_STATE; }
int sgb_batch_step_ensemble(sgb_batch*, double, double, uint64_t, int32_t, int32_t, int64_t*) { return SGB_ERR_STATE; }
int sgb_batch_event_record(sgb_batch*, int32_t) { return SGB_ERR_STATE; }
int sgb_batch_event_elapsed(sgb_batch*, int32_t, int32_t, float*) { return SGB_ERR_STATE; }
int64_t sgb_batch_kernel_launches(const sgb_batch*) { return 0; }

}  // extern "C"
