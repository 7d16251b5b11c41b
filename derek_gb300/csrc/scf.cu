// SCF driver (placeholder entry points until the subspace solver lands).
#include "handle.h"

extern "C" int derek_scf_alloc(derek_gpu_t *) { return DEREK_OK; }
extern "C" void derek_scf_free(derek_gpu_t *) {}

extern "C" {
int derek_gpu_overlap(derek_gpu_t *, int, int, double *) { return DEREK_ERR_UNSUPPORTED; }
int derek_gpu_scf_iterate(derek_gpu_t *, derek_scf_report *) { return DEREK_ERR_UNSUPPORTED; }
int derek_gpu_scf_run(derek_gpu_t *, int, double, derek_scf_report *) { return DEREK_ERR_UNSUPPORTED; }
int derek_gpu_get_eigenvalues(derek_gpu_t *, int, double *) { return DEREK_ERR_UNSUPPORTED; }
int derek_gpu_get_occupations(derek_gpu_t *, int, double *) { return DEREK_ERR_UNSUPPORTED; }
int derek_gpu_get_density(derek_gpu_t *, int, double *) { return DEREK_ERR_UNSUPPORTED; }
}
