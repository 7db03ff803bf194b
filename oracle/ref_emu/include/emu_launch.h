// Kernel-launch and __syncthreads emulation for running the reference's CUDA
// sources on the CPU (TEST INFRASTRUCTURE ONLY).  The build recipe rewrites
// every `kernel<<<grid, block, smem>>>(args)` of the reference into
// `EMU_LAUNCH(kernel, grid, block, smem)(args)`; the grid then runs
// synchronously on the host, one block after another.  Kernels that call
// __syncthreads run their threads as cooperative fibers (ucontext), so a
// barrier switches to the next thread of the block.
#pragma once

#include <cstddef>

#include "cuda_runtime.h"

namespace emu {

void syncthreads();
void run_grid(const char* name, dim3 grid, dim3 block, void (*thunk)(void*), void* ctx);

template <class F>
struct Launch {
    const char* name;
    F f;
    dim3 grid, block;
    template <class... A>
    void operator()(A... args)
    {
        auto call = [&]() { f(args...); };
        using Call = decltype(call);
        run_grid(name, grid, block, [](void* p) { (*static_cast<Call*>(p))(); }, &call);
    }
};

template <class F>
Launch<F> launcher(const char* name, F f, dim3 grid, dim3 block, size_t = 0, cudaStream_t = 0)
{
    return Launch<F>{name, f, grid, block};
}

}  // namespace emu

#define __syncthreads() ::emu::syncthreads()
#define EMU_LAUNCH(k, ...) ::emu::launcher(#k, [&](auto&&... a_) { k(a_...); }, __VA_ARGS__)
