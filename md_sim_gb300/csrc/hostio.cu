// Host <-> device transfers of the drop-in calls (mdg_force_get, mdg_shake).
//
// Pinned host memory is mapped into the GPU's address space; on a Grace-Blackwell node the GPU
// reaches it over the coherent NVLink-C2C link.  A call moves a dozen or more separate arrays
// (positions, offsets, centres in; forces, torques, energies, status out), and one DMA copy per
// array costs a few microseconds of setup latency each, serialised on the stream.  Here every
// array whose host side is pinned joins one batch that a single kernel copies (one CTA column per
// array, 8-byte words, so the bits move unchanged); the others go through cudaMemcpyAsync.

#include <map>
#include <mutex>

#include "ctx.h"

namespace mdg {

namespace {

// Ranges pinned through mdg_pin_host: base -> (bytes, the GPU's address of base).  They stay
// valid until mdg_unpin_host, so a call finds its arrays here without asking the driver.
std::mutex g_pin_mu;
std::map<uintptr_t, std::pair<size_t, uintptr_t>> g_pinned;

void* registry_address(const void* p) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pinned.upper_bound(a);
    if (it == g_pinned.begin()) return nullptr;
    --it;
    if (a - it->first >= it->second.first) return nullptr;
    return reinterpret_cast<void*>(it->second.second + (a - it->first));
}

__global__ void k_io_copy(IoBatch b) {
    const int s = blockIdx.y;
    const unsigned long long* __restrict__ src = b.src[s];
    unsigned long long* __restrict__ dst = b.dst[s];
    const long n = b.n[s];
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// The GPU's address of a host array, or nullptr when the array is not pinned (pageable memory
// is copied through the driver's staging instead).
void* mapped_address(const void* p) {
    if (void* r = registry_address(p)) return r;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // some drivers report memory CUDA does not know as an error: clear it
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

}  // namespace

cudaError_t io_add(Ctx& c, IoBatch& b, void* dst, const void* src, long nwords, bool h2d) {
    if (nwords <= 0 || !dst || !src) return cudaSuccess;
    if (b.nseg < IoBatch::kMax) {
        void* m = mapped_address(h2d ? src : dst);
        if (m) {
            b.src[b.nseg] = static_cast<const unsigned long long*>(h2d ? m : src);
            b.dst[b.nseg] = static_cast<unsigned long long*>(h2d ? dst : m);
            b.n[b.nseg] = nwords;
            b.nmax = std::max(b.nmax, nwords);
            ++b.nseg;
            return cudaSuccess;
        }
    }
    return cudaMemcpyAsync(dst, src, sizeof(unsigned long long) * nwords,
                           h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c.stream);
}

cudaError_t pin_host_range(void* p, size_t bytes) {
    cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
    if (e != cudaSuccess) return e;
    void* d = nullptr;
    e = cudaHostGetDevicePointer(&d, p, 0);
    if (e != cudaSuccess) {
        cudaHostUnregister(p);
        return e;
    }
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pinned[reinterpret_cast<uintptr_t>(p)] = {bytes, reinterpret_cast<uintptr_t>(d)};
    return cudaSuccess;
}

cudaError_t unpin_host_range(void* p) {
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        g_pinned.erase(reinterpret_cast<uintptr_t>(p));
    }
    return cudaHostUnregister(p);
}

void io_flush(Ctx& c, IoBatch& b) {
    if (b.nseg == 0) return;
    const int gx = (int)std::min<long>((b.nmax + 255) / 256, 32);
    k_io_copy<<<dim3(gx, b.nseg), 256, 0, c.stream>>>(b);
    b.nseg = 0;
    b.nmax = 0;
}

}  // namespace mdg
