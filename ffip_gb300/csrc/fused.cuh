// Fused H+E z-marching pass (placeholder until the fused kernel lands).
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>

#include "engine.hpp"

namespace ffipg
{
template <typename T>
inline void launch_fused(const FusedParams<T> &, cudaStream_t)
{
    throw std::runtime_error("fused pass not built");
}
} // namespace ffipg
