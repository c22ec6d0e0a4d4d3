// Placeholder until the tcgen05 engine lands.
#include "sb_host.h"
#include "sb_internal.h"
namespace sbk {
struct TcEngine { int dtype; };
sb_status tc_create(TcEngine **, const TcSetup &, const float *, int, std::string &err, cudaStream_t) { err = "tensor-core path not built"; return SB_ERR_UNSUPPORTED; }
void tc_destroy(TcEngine *e) { delete e; }
int64_t tc_footprint(const TcSetup &) { return 0; }
cudaError_t tc_prepare(TcEngine *, const float *, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t tc_step(TcEngine *, int, float *, float *, const float *, float, float, float, float, double *, uint32_t *, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t tc_energy(TcEngine *, int, const float *, const float *, double *, uint32_t *, cudaStream_t) { return cudaErrorNotSupported; }
int tc_dtype(const TcEngine *e) { return e ? e->dtype : 0; }
}
