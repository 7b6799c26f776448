// Instantiates the (radius 1..4) kernels for float field storage.
#include "ofd_impl.cuh"
namespace ofd {
Backend *make_backend_f32(int R) { return make_backend_t<float>(R); }
}  // namespace ofd
