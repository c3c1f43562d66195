// Stand-ins for the library's error reporting and device entry points, so that the host file readers
// (csrc/h5.cpp, csrc/mm.cpp) build alone under AddressSanitizer and UBSan (tests/test_readers_sanitized.py).
// The device entry points the readers reach (converting a loaded CSR5 group, exporting one to store)
// return an error here.
#include <cstdarg>
#include <cstdio>

#include "internal.hpp"
namespace dimgpu {
static thread_local char g_msg[1024];
void set_error(const char* fmt, ...) {
    va_list a;
    va_start(a, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, a);
    va_end(a);
}
int fail(int code, const char* fmt, ...) {
    va_list a;
    va_start(a, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, a);
    va_end(a);
    return code;
}
int cuda_fail(cudaError_t, const char*) { return DIMGPU_ERR_CUDA; }
}  // namespace dimgpu
extern "C" {
const char* dimgpu_last_error_string(void) { return dimgpu::g_msg; }
int dimgpu_csr5_from_csr(uint32_t, uint32_t, uint64_t, const uint32_t*, const uint32_t*, const double*, int,
                         const dimgpu_csr5_options*, void*, dimgpu_csr5** out) {
    if (out)
        *out = nullptr;
    return DIMGPU_ERR_CUDA;
}
int dimgpu_csr5_get_info(const dimgpu_csr5*, dimgpu_csr5_info*) { return DIMGPU_ERR_CUDA; }
int dimgpu_csr5_export(const dimgpu_csr5*, uint32_t*, void*, uint32_t*, uint32_t*, double*, uint32_t*, uint32_t*) {
    return DIMGPU_ERR_CUDA;
}
}  // extern "C"
