// scan_ws.cu — single-document instantiations of the warp-specialised scan kernel
// (scan_ws_kernel.cuh) and its launch parameters.
#include "scan_ws_kernel.cuh"

namespace pars {

#define PARS_INST(P, B) \
	template __global__ void k_scan_ws<P, B, false>(const WsArgs, const __grid_constant__ CUtensorMap);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
PARS_INST(kPathEscape, false)
PARS_INST(kPathEscape, true)
#undef PARS_INST

int scan_ws_threads() {
	return kWsThreads;
}

int scan_ws_smem_bytes() {
	return SmemWs::kBytes;
}

// The fold window of a tile (G - 1 aggregates) is held by one warp, kLB per lane.
int scan_ws_max_grid() {
	return 32 * kLB;
}

int scan_ws_tile_bytes() {
	return kWsTile;
}

const void* scan_ws_kernel(int path, bool brackets) {
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, false, false>);
		case 1: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, true, false>);
		case 2: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, false, false>);
		case 3: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, true, false>);
		case 4: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, false, false>);
		case 5: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, true, false>);
		case 6: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, false, false>);
		case 7: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, true, false>);
		default: return nullptr;
	}
}

}  // namespace pars
