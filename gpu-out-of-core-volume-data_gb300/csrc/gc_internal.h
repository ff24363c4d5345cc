// Internal helpers shared by the translation units of libgcgb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <new>
#include <stdexcept>
#include <string>

#include "gc_gb300.h"

namespace gc {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_error(const std::string &msg);
void clear_error();

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error(code, msg); }

inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fail(GC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define GC_CUDA(x) ::gc::check_cuda((x), #x)
#define GC_REQUIRE(cond, msg)                                  \
    do {                                                       \
        if (!(cond)) ::gc::fail(GC_ERR_INVALID, (msg));        \
    } while (0)

// Runs f and converts exceptions into a status code + thread-local message.
template <class F>
int guard(F &&f) {
    try {
        clear_error();
        f();
        return GC_OK;
    } catch (const Error &e) {
        set_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return GC_ERR_NOMEM;
    } catch (const std::exception &e) {
        set_error(e.what());
        return GC_ERR_INVALID;
    }
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline uint32_t div_up(uint64_t a, uint64_t b) { return static_cast<uint32_t>((a + b - 1) / b); }

// Counts kernel launches (gc_kernel_launches).
void count_launch(uint32_t n = 1);

// Number of SMs of the current device (cached per process for device 0..7).
int sm_count();

// Validation of a volume description; throws GC_ERR_INVALID.
void validate_volume(const gc_volume_desc &v);
inline uint32_t channel_bytes(const gc_volume_desc &v) { return v.encoded_bytes / v.channels; }

}  // namespace gc
