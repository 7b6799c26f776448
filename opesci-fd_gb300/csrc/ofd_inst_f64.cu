// Instantiates the (radius 1..4) kernels for double field storage.
#include "ofd_impl.cuh"
namespace ofd {
Backend *make_backend_f64(int R) { return make_backend_t<double>(R); }
}  // namespace ofd
