// cnv_guard.h -- guard regions around device buffers, for the testing-only config field
// test_guard_cells: out-of-bounds writes are found without a sanitizer.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>
#include <vector>

namespace cnv {

// While `on`, alloc() puts kGuardBytes of 0xFF bytes (a NaN in every lane width) before and after
// each buffer, and check() compares every guard region with that pattern; while off, alloc() is a
// plain cudaMalloc. 4096 bytes keep the buffer's 256-byte alignment.
class GuardSet {
  public:
    static constexpr size_t kGuardBytes = 4096;
    bool on = false;

    cudaError_t alloc(void** p, size_t bytes, const char* name);
    // cudaFree of a pointer alloc() returned (or of any other device pointer); null is ignored
    void release(void* p);
    // true if every guard region still holds 0xFF; else false, with *what naming the region.
    // Synchronous (waits for the device): call it after the work that might have written there.
    bool check(std::string* what) const;
    // change one byte of the guard after the named buffer: the checker's own test
    cudaError_t plant(const char* name) const;

  private:
    struct Buf {
        char* base;
        size_t bytes;
        std::string name;
    };
    std::vector<Buf> bufs_;
};

}  // namespace cnv
