// h2w_matvec_static: the block-row GEMV matvec with its workspace in a
// file-scope device array, so that a call allocates nothing.
//
// The array holds H2W_STATIC_WS_DOUBLES doubles (16 MiB) of workspace rows
// (an FP32 product uses them as twice as many floats), followed by the grid
// barrier state and the barrier's error word. Its device address is looked
// up once per device, on the first call on that device, with that device
// current (cudaGetSymbolAddress); later calls reuse it (the cached address
// does not survive a cudaDeviceReset of that device). Every call clears the
// workspace rows it uses, the barrier state and the error word before its
// launch, and reads the error word back once the product has finished, so a
// grid-barrier wait that ran out fails that call with H2W_ERR_CUDA. All
// handles and all calls on a device share the one array and it keeps the
// last call's contents, so calls whose kernels overlap on the GPU (two
// streams, two host threads) race on it: serialise them.
#include <mutex>
#include <string>

#include "../../include/h2w.h"
#include "kernels.cuh"

namespace h2w {
int handle_device(const h2w_handle *h);
int handle_fail(h2w_handle *h, int code, const char *msg);
int matvec_external_ws(h2w_handle *h, const double *x, double *y, int precision, void *stream, double *ws,
                       int64_t ws_cap, unsigned *bar, int32_t *err);
}  // namespace h2w

namespace {

constexpr int64_t H2W_STATIC_WS_DOUBLES = int64_t(1) << 21;  // 16 MiB of workspace rows
constexpr int64_t H2W_STATIC_TAIL = 32;                      // barrier state + error word (256 bytes)
constexpr int H2W_MAX_DEVICES = 64;

static __device__ __align__(256) double h2w_static_scratch[H2W_STATIC_WS_DOUBLES + H2W_STATIC_TAIL];

std::mutex g_mu;
double *g_ptr[H2W_MAX_DEVICES] = {};

// Device address of the array on `dev` (set-up on the first call per device).
cudaError_t static_scratch(int dev, double **out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
        int cur = -1;
        cudaError_t e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return e;
        if (cur != dev && (e = cudaSetDevice(dev)) != cudaSuccess) return e;
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, h2w_static_scratch);
        if (cur != dev) cudaSetDevice(cur);
        if (e != cudaSuccess) return e;
        g_ptr[dev] = p;
    }
    *out = g_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int h2w_matvec_static(h2w_handle *h, const double *x, double *y, int precision, void *stream) {
    if (!h) return H2W_ERR_ARG;
    const int dev = h2w::handle_device(h);
    if (dev < 0) return h2w::handle_fail(h, H2W_ERR_STATE, "host-only handle (device < 0) has no operator");
    if (dev >= H2W_MAX_DEVICES) return h2w::handle_fail(h, H2W_ERR_ARG, "device ordinal beyond the static table");
    double *ws = nullptr;
    const cudaError_t e = static_scratch(dev, &ws);
    if (e != cudaSuccess) {
        const std::string m = std::string("cudaGetSymbolAddress of the static workspace: ") + cudaGetErrorString(e);
        return h2w::handle_fail(h, H2W_ERR_CUDA, m.c_str());
    }
    unsigned *bar = reinterpret_cast<unsigned *>(ws + H2W_STATIC_WS_DOUBLES);
    int32_t *err = reinterpret_cast<int32_t *>(ws + H2W_STATIC_WS_DOUBLES + 1);
    return h2w::matvec_external_ws(h, x, y, precision, stream, ws, H2W_STATIC_WS_DOUBLES, bar, err);
}
