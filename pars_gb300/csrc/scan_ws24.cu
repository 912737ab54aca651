// scan_ws24.cu — single-document instantiations of the warp-specialised scan kernel
// (scan_ws_kernel.cuh) with 24 workers: 48 KiB tiles, 800 threads, two TMA boxes
// per tile.  More resident warps hide more latency on long documents.
#include "scan_ws_kernel.cuh"

namespace pars {

#define PARS_INST(P, B) \
	template __global__ void k_scan_ws<P, B, false, 24>(const WsArgs, const __grid_constant__ CUtensorMap);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
PARS_INST(kPathEscape, false)
PARS_INST(kPathEscape, true)
#undef PARS_INST

const void* scan_ws24_kernel(int path, bool brackets) {
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, false, false, 24>);
		case 1: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, true, false, 24>);
		case 2: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, false, false, 24>);
		case 3: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, true, false, 24>);
		case 4: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, false, false, 24>);
		case 5: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, true, false, 24>);
		case 6: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, false, false, 24>);
		case 7: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, true, false, 24>);
		default: return nullptr;
	}
}

}  // namespace pars
