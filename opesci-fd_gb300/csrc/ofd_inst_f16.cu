// The kernels of one radius (OFD_INST_R, 1..4) for __half field storage; the
// build compiles this unit once per radius.
#include "ofd_impl.cuh"
#ifndef OFD_INST_R
#error "compile with -DOFD_INST_R=1, 2, 3 or 4"
#endif
namespace ofd {
OFD_DEFINE_BACKEND(__half)
}  // namespace ofd
