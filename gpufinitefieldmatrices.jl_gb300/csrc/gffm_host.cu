// gffm_host.cu -- library-wide host plumbing: error reporting, device checks,
// scratch allocation and the device-side error word.
#include "gffm_common.cuh"

#include <cstring>
#include <mutex>

#define GFFM_VERSION_STRING "gffm-gb300 0.1.0 (sm_103a)"

// One word per device; kernels OR a code into it when a bounded wait gives up.
static __device__ int g_device_error;

namespace gffm {

static thread_local char tl_msg[512] = "";

int set_error(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(tl_msg, sizeof(tl_msg), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_error(cudaError_t e, const char *what) {
    return set_error(GFFM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

cudaStream_t as_stream(gffm_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

static thread_local ProfileHook tl_hook;
ProfileHook &profile_hook() { return tl_hook; }

namespace {
constexpr int kMaxDevices = 64;
struct DevInfo {
    int ok = -1;       // -1 unknown, else gffm status
    int sms = 0;
    int *err = nullptr;
};
DevInfo g_dev[kMaxDevices];
std::mutex g_mu;

DevInfo *dev_info(int *status) {
    int d = 0;
    cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) {
        *status = cuda_error(e, "cudaGetDevice");
        return nullptr;
    }
    if (d < 0 || d >= kMaxDevices) {
        *status = set_error(GFFM_ERR_UNSUPPORTED, "device ordinal %d out of range", d);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    DevInfo &di = g_dev[d];
    if (di.ok < 0) {
        int major = 0, minor = 0, sms = 0;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
        di.sms = sms;
        if (!(major == 10 && minor == 3)) {
            di.ok = GFFM_ERR_UNSUPPORTED;
        } else {
            void *p = nullptr;
            cudaError_t e2 = cudaGetSymbolAddress(&p, g_device_error);
            if (e2 != cudaSuccess) {
                *status = cuda_error(e2, "cudaGetSymbolAddress(error word)");
                return nullptr;
            }
            di.err = static_cast<int *>(p);
            di.ok = GFFM_OK;
        }
    }
    if (di.ok != GFFM_OK) {
        *status = set_error(di.ok, "libgffm kernels are built for sm_103a (GB300); this device is not sm_103");
        return nullptr;
    }
    *status = GFFM_OK;
    return &di;
}
}  // namespace

int check_device() {
    int st;
    return dev_info(&st) ? GFFM_OK : st;
}

int sm_count() {
    int st;
    DevInfo *di = dev_info(&st);
    return di ? di->sms : 0;
}

int *device_error_flag() {
    int st;
    DevInfo *di = dev_info(&st);
    return di ? di->err : nullptr;
}

int Scratch::acquire(void *ws, size_t ws_bytes, size_t need, cudaStream_t s) {
    stream = s;
    if (need == 0) return GFFM_OK;
    if (ws != nullptr) {
        if (ws_bytes < need)
            return set_error(GFFM_ERR_WORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes needed",
                             ws_bytes, need);
        if ((reinterpret_cast<uintptr_t>(ws) & 255u) != 0)
            return set_error(GFFM_ERR_ARG, "workspace must be 256-byte aligned");
        ptr = ws;
        return GFFM_OK;
    }
    cudaError_t e = cudaMallocAsync(&ptr, need, s);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return cuda_error(e, "cudaMallocAsync(workspace)");
    }
    owned = true;
    return GFFM_OK;
}

Scratch::~Scratch() {
    if (owned && ptr) cudaFreeAsync(ptr, stream);
}

}  // namespace gffm

extern "C" {

const char *gffm_version(void) { return GFFM_VERSION_STRING; }

const char *gffm_last_error_string(void) { return gffm::tl_msg; }

int gffm_device_status(gffm_stream_t stream) {
    int *flag = gffm::device_error_flag();
    if (!flag) return gffm::check_device();
    int h = 0;
    GFFM_CUDA(cudaStreamSynchronize(gffm::as_stream(stream)));
    GFFM_CUDA(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (h != 0) {
        int zero = 0;
        GFFM_CUDA(cudaMemcpy(flag, &zero, sizeof(int), cudaMemcpyHostToDevice));
        return gffm::set_error(GFFM_ERR_TIMEOUT, "a device-side wait gave up (code %d); results are invalid", h);
    }
    return GFFM_OK;
}

int gffm_profile_next_kernel(void *start_event, void *stop_event) {
    gffm::profile_hook().start = static_cast<cudaEvent_t>(start_event);
    gffm::profile_hook().stop = static_cast<cudaEvent_t>(stop_event);
    return GFFM_OK;
}

int gffm_find_max_stripe_ops(int bits, int64_t N, int64_t *out) {
    if (!out) return gffm::set_error(GFFM_ERR_ARG, "out is NULL");
    if (bits != 53 && bits != 24 && bits != 11)
        return gffm::set_error(GFFM_ERR_ARG, "bits must be 53, 24 or 11 (Float64/32/16)");
    if (N < 1) return gffm::set_error(GFFM_ERR_MODULUS, "modulus %lld < 1", (long long)N);
    if (N == 1) {
        *out = INT64_MAX;
        return GFFM_OK;
    }
    // floor((2^bits - 1) / (N-1)^2) - 1 with exact integer arithmetic
    unsigned __int128 num = ((unsigned __int128)1 << bits) - 1;
    unsigned __int128 den = (unsigned __int128)(N - 1) * (unsigned __int128)(N - 1);
    *out = (int64_t)(num / den) - 1;
    return GFFM_OK;
}

}  // extern "C"
