// sdpd.cu — SDPD particle step (placeholder until the flow kernels land).
#include "sdpd.cuh"

namespace spg {
struct SdpdState { int dummy; };
SdpdState* sdpd_create(const sp_scenario&, int, cudaStream_t, std::string* err) {
    *err = "moving domains are not supported yet";
    return nullptr;
}
void sdpd_destroy(SdpdState* s) { delete s; }
int sdpd_advance(SdpdState*, int, double*, long long*, std::string* err) {
    *err = "moving domains are not supported yet";
    return SP_E_UNSUPPORTED;
}
int sdpd_get_state(SdpdState*, double*, double*, double*, std::string* err) {
    *err = "moving domains are not supported yet";
    return SP_E_UNSUPPORTED;
}
int sdpd_copy_neighbors(SdpdState*, int, int*, int*, double*, double*, double*, std::string* err) {
    *err = "moving domains are not supported yet";
    return SP_E_UNSUPPORTED;
}
}  // namespace spg
