// Instantiates the (radius 1..4) kernels for __half field storage.
#include "ofd_impl.cuh"
namespace ofd {
Backend *make_backend_f16(int R) { return make_backend_t<__half>(R); }
}  // namespace ofd
