// Instantiates the (radius 1..4) kernels for __nv_bfloat16 field storage.
#include "ofd_impl.cuh"
namespace ofd {
Backend *make_backend_bf16(int R) { return make_backend_t<__nv_bfloat16>(R); }
}  // namespace ofd
