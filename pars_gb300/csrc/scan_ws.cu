// scan_ws.cu — single-document instantiations of the warp-specialised scan kernel
// (scan_ws_kernel.cuh) with 16 workers, and the launch parameters of every tile
// shape (the 24-worker kernels are in scan_ws24.cu).
#include "scan_ws_kernel.cuh"

namespace pars {

#define PARS_INST(P, B) \
	template __global__ void k_scan_ws<P, B, false, 16>(const WsArgs, const __grid_constant__ CUtensorMap);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
PARS_INST(kPathEscape, false)
PARS_INST(kPathEscape, true)
#undef PARS_INST

static_assert(kWsShapeWorkers[0] == 16 && kWsShapeWorkers[1] == 24, "shape table");

int scan_ws_threads(int shape) {
	return shape ? WsGeom<24>::kThreads : WsGeom<16>::kThreads;
}

int scan_ws_smem_bytes(int shape) {
	return shape ? SmemWsT<24>::kBytes : SmemWsT<16>::kBytes;
}

// The fold window of a tile (G - 1 aggregates) is held by one warp, kLB per lane.
int scan_ws_max_grid() {
	return 32 * kLB;
}

int scan_ws_tile_bytes(int shape) {
	return shape ? WsGeom<24>::kTile : WsGeom<16>::kTile;
}

int scan_ws_box_rows(int shape) {
	return shape ? WsGeom<24>::kBoxRows : WsGeom<16>::kBoxRows;
}

const void* scan_ws24_kernel(int path, bool brackets);

const void* scan_ws_kernel(int path, bool brackets, int shape) {
	if (shape)
		return scan_ws24_kernel(path, brackets);
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, false, false, 16>);
		case 1: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, true, false, 16>);
		case 2: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, false, false, 16>);
		case 3: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, true, false, 16>);
		case 4: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, false, false, 16>);
		case 5: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, true, false, 16>);
		case 6: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, false, false, 16>);
		case 7: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, true, false, 16>);
		default: return nullptr;
	}
}

}  // namespace pars
