// sgb_static.cu -- sgb_energy_grad_static: the energy gradient without any device
// allocation.
//
// sgb_energy_grad evaluates the gradient into a device scratch buffer that the handle
// grows with cudaMalloc on first use. Some callers cannot allow that: a host that runs
// under a fixed device-memory budget owned by its own pool allocator, or a real-time loop
// that must not enter the CUDA allocator. This variant writes the gradient into a
// file-scope static device array instead, so a call performs no allocation of any kind.
//
// Limits and sharing rules:
//   - The array holds SGB_STATIC_GRAD_DOUBLES (2^20) doubles, 8 MiB, resident on every
//     device that loads the library until the process exits. A gradient needs 3 doubles
//     per site in dipole modes and 2N per site in SU(N) mode, so at most 349,525 dipole
//     sites (174,762 SU(3) sites); larger systems get SGB_ERR_ARG.
//   - Every call, from every handle on that device, shares the one array and it keeps the
//     previous call's contents. The gradient kernel overwrites every element it returns,
//     so nothing needs clearing, but calls whose kernels overlap on the GPU race: issue
//     them on one thread, one after the other (each call waits for its own copy-out).
//   - The first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (with that device current). Make that first call before any
//     stream capture begins.
#include <mutex>
#include <string>
#include "sgb_handles.h"

#define SGB_STATIC_GRAD_DOUBLES (1 << 20)
#define SGB_STATIC_MAX_DEVICES 64

static __device__ __align__(256) double sgb_static_grad_scratch[SGB_STATIC_GRAD_DOUBLES];

namespace {
std::mutex g_static_mu;
double* g_static_ptr[SGB_STATIC_MAX_DEVICES] = {};

// Device address of the scratch array on `device`, resolved once per device.
cudaError_t static_scratch(int device, double** out) {
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (device < 0 || device >= SGB_STATIC_MAX_DEVICES) return cudaErrorInvalidDevice;
    if (!g_static_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, sgb_static_grad_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[device] = static_cast<double*>(p);
    }
    *out = g_static_ptr[device];
    return cudaSuccess;
}
}  // namespace

extern "C" int sgb_energy_grad_static(sgb_system* s, double* grad) {
    if (!s || !grad) return SGB_ERR_ARG;
    const size_t n = s->sun ? (size_t)2 * s->N * s->ns : (size_t)3 * s->ns;
    if (n > SGB_STATIC_GRAD_DOUBLES) {
        s->err = "sgb_energy_grad_static: the gradient needs " + std::to_string(n) +
                 " doubles but the static scratch holds " + std::to_string(SGB_STATIC_GRAD_DOUBLES) +
                 "; use sgb_energy_grad for this system";
        return SGB_ERR_ARG;
    }
    if (!s->state_set || s->tables_dirty || !s->tables) {
        s->err = "sgb_energy_grad_static: set the state (sgb_set_state) after the last coupling change first";
        return SGB_ERR_STATE;
    }
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e == cudaSuccess && cur != s->d.device) e = cudaSetDevice(s->d.device);
    double* scratch = nullptr;
    if (e == cudaSuccess) e = static_scratch(s->d.device, &scratch);
    if (e != cudaSuccess) {
        s->err = std::string("sgb_energy_grad_static: ") + cudaGetErrorString(e);
        return SGB_ERR_CUDA;
    }
    int rc;
    if (!s->sun) {
        rc = s->fp32 ? dip_launch_grad<float>(s->mf, (const float*)s->S, scratch, s->stream)
                     : dip_launch_grad<double>(s->md, (const double*)s->S, scratch, s->stream);
    } else {
        rc = s->fp32 ? sun_launch_grad<float>(s->mf, (const float*)s->Z, (const float*)s->S, (const float*)s->Q, scratch, s->stream)
                     : sun_launch_grad<double>(s->md, (const double*)s->Z, (const double*)s->S, (const double*)s->Q, scratch, s->stream);
    }
    s->launches++;
    if (rc == SGB_OK) {
        e = cudaMemcpyAsync(grad, scratch, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = SGB_ERR_CUDA;
    } else {
        e = cudaGetLastError();
    }
    if (rc != SGB_OK) {
        s->err = std::string("sgb_energy_grad_static: ") + cudaGetErrorString(e);
        return rc;
    }
    return SGB_OK;
}
