// Tiled sweeps (placeholder until the TMA kernels land).
#pragma once
#include "ofd_common.cuh"
namespace ofd {
template <int R, typename S> bool tiled_supported(const Geom &) { return false; }
template <int R, typename S> void launch_stress_tiled(const SweepArgs<S> &, cudaStream_t) {}
template <int R, typename S> void launch_velocity_tiled(const SweepArgs<S> &, cudaStream_t) {}
}  // namespace ofd
