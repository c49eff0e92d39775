// cnv_guard.cpp -- guard regions around device buffers (see cnv_guard.h).
#include "cnv_guard.h"

namespace cnv {

cudaError_t GuardSet::alloc(void** p, size_t bytes, const char* name) {
    if (!on) return cudaMalloc(p, bytes);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&base), bytes + 2 * kGuardBytes);
    if (e != cudaSuccess) return e;
    e = cudaMemset(base, 0xFF, kGuardBytes);
    if (e == cudaSuccess) e = cudaMemset(base + kGuardBytes + bytes, 0xFF, kGuardBytes);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // the guards are in place before any use
    if (e != cudaSuccess) {
        cudaFree(base);
        return e;
    }
    bufs_.push_back(Buf{base, bytes, name});
    *p = base + kGuardBytes;
    return cudaSuccess;
}

void GuardSet::release(void* p) {
    if (!p) return;
    for (auto& b : bufs_)
        if (b.base && b.base + kGuardBytes == p) {
            cudaFree(b.base);
            b.base = nullptr;
            return;
        }
    cudaFree(p);
}

bool GuardSet::check(std::string* what) const {
    if (bufs_.empty()) return true;
    if (cudaDeviceSynchronize() != cudaSuccess) {
        if (what) *what = "device synchronisation before the guard check failed";
        return false;
    }
    std::vector<unsigned char> h(kGuardBytes);
    for (const auto& b : bufs_) {
        if (!b.base) continue;
        for (int after = 0; after < 2; ++after) {
            const char* src = after ? b.base + kGuardBytes + b.bytes : b.base;
            if (cudaMemcpy(h.data(), src, kGuardBytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
                if (what) *what = "guard copy failed";
                return false;
            }
            for (size_t k = 0; k < kGuardBytes; ++k)
                if (h[k] != 0xFF) {
                    if (what)
                        *what = std::string("guard bytes ") + (after ? "after " : "before ") + b.name +
                                " changed (byte " + std::to_string(k) + " of " + std::to_string(kGuardBytes) + ")";
                    return false;
                }
        }
    }
    return true;
}

cudaError_t GuardSet::plant(const char* name) const {
    for (const auto& b : bufs_)
        if (b.base && b.name == name) {
            cudaError_t e = cudaMemset(b.base + kGuardBytes + b.bytes, 0, 1);
            return e == cudaSuccess ? cudaDeviceSynchronize() : e;
        }
    return cudaErrorInvalidValue;
}

}  // namespace cnv
