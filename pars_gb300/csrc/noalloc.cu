// noalloc.cu — the fixed device scratch behind pars_scan_device_noalloc.
//
// Some callers cannot allocate on their scan path: a serving loop whose latency
// budget cannot absorb cudaMalloc / cudaFree (both may wait for the whole device),
// or a host framework that owns every byte of device memory through its own pool
// and forbids allocations it does not track.  For them the scan's scratch (result
// block, tile counters, look-back descriptors) lives in one array compiled into
// the library, so the call itself allocates nothing.  The array is shared by every
// context on a device: calls that overlap in time race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "pars_gb300.h"
#include "pars_internal.h"

namespace pars {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Copies the scan's result block into the caller's result record.
__global__ void k_noalloc_finish(const DevResult* r, pars_noalloc_result* out) {
	out->n_struct	   = r->n_struct;
	out->unclosed_mode = static_cast<std::int32_t>(r->unclosed);
	out->status		   = r->error ? PARS_ETIMEDOUT : 0;
}

const void* noalloc_finish_kernel() {
	return reinterpret_cast<const void*>(&k_noalloc_finish);
}

// Device address of the scratch on the current device, looked up once per device.
cudaError_t noalloc_scratch(int device, unsigned char** addr) {
	constexpr int			kMaxDevices = 64;
	static std::mutex		mu;
	static unsigned char*	cache[kMaxDevices] = {};
	if (device < 0 || device >= kMaxDevices)
		return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> lock(mu);
	if (!cache[device]) {
		void*			  p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess)
			return e;
		cache[device] = static_cast<unsigned char*>(p);
	}
	*addr = cache[device];
	return cudaSuccess;
}

}  // namespace pars
