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
//   - With dipole-dipole interactions enabled the long-range term is included, as in
//     sgb_energy_grad. It runs on the transforms and buffers that sgb_set_dipole_dipole
//     allocated, so it allocates nothing either. In SU(N) mode the term needs 3 more
//     doubles per site of the array for dE/dS at the expected dipoles (at most 116,508
//     SU(3) sites with dipole-dipole interactions).
//   - The caller's current device is the same after the call as before it.
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

namespace {
// Makes `device` current for the lifetime of the guard and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int device) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != device) err = cudaSetDevice(device);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

template <class R> const Model<R>& model_of(const sgb_system* s);
template <> const Model<float>& model_of<float>(const sgb_system* s) { return s->mf; }
template <> const Model<double>& model_of<double>(const sgb_system* s) { return s->md; }

template <class R>
int static_grad(sgb_system* s, double* scratch) {
    const Model<R>& M = model_of<R>(s);
    if (!s->sun) {
        int rc = dip_launch_grad<R>(M, (const R*)s->S, scratch, s->stream);
        s->launches++;
        if (rc == SGB_OK && s->ewald_on) {
            rc = ewald_apply<R>(s->ew, (const R*)s->S, scratch, nullptr, s->stream);
            s->launches += 4;
        }
        return rc;
    }
    int rc = sun_launch_grad<R>(M, (const R*)s->Z, (const R*)s->S, (const R*)s->Q, scratch, s->stream);
    s->launches++;
    if (rc == SGB_OK && s->ewald_on) {
        // dE/dS of the dipole-dipole term at the expected dipoles, in the array after HZ
        double* f = scratch + (size_t)2 * s->N * s->ns;
        if (cudaMemsetAsync(f, 0, sizeof(double) * 3 * (size_t)s->ns, s->stream) != cudaSuccess) return SGB_ERR_CUDA;
        rc = ewald_apply<R>(s->ew, (const R*)s->S, f, nullptr, s->stream);
        s->launches += 4;
        if (rc == SGB_OK) rc = sun_launch_add_dipole_field<R>(M, (const R*)s->Z, f, scratch, s->stream);
        s->launches++;
    }
    return rc;
}
}  // namespace

extern "C" int sgb_energy_grad_static(sgb_system* s, double* grad) {
    if (!s || !grad) return SGB_ERR_ARG;
    const size_t n = s->sun ? (size_t)2 * s->N * s->ns : (size_t)3 * s->ns;
    const size_t need = n + (s->sun && s->ewald_on ? (size_t)3 * s->ns : 0);
    if (need > SGB_STATIC_GRAD_DOUBLES) {
        s->err = "sgb_energy_grad_static: the gradient needs " + std::to_string(need) +
                 " doubles but the static scratch holds " + std::to_string(SGB_STATIC_GRAD_DOUBLES) +
                 "; use sgb_energy_grad for this system";
        return SGB_ERR_ARG;
    }
    if (!s->state_set || s->tables_dirty || !s->tables) {
        s->err = "sgb_energy_grad_static: set the state (sgb_set_state) after the last coupling change first";
        return SGB_ERR_STATE;
    }
    DeviceGuard dev(s->d.device);
    cudaError_t e = dev.err;
    double* scratch = nullptr;
    if (e == cudaSuccess) e = static_scratch(s->d.device, &scratch);
    if (e != cudaSuccess) {
        s->err = std::string("sgb_energy_grad_static: ") + cudaGetErrorString(e);
        return SGB_ERR_CUDA;
    }
    int rc = s->fp32 ? static_grad<float>(s, scratch) : static_grad<double>(s, scratch);
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
