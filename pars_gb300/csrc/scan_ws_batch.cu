// scan_ws_batch.cu — batch instantiations of the warp-specialised scan kernel
// (scan_ws_kernel.cuh): many documents in one persistent launch, each CTA scanning
// whole documents, the running prefix reset at every document's first tile.  The
// batch kernel runs 16 workers (tile shape 0): a small document costs a tile pass.
#include "scan_ws_kernel.cuh"

namespace pars {

#define PARS_INST(P, B) \
	template __global__ void k_scan_ws<P, B, true, 16>(const WsArgs, const __grid_constant__ CUtensorMap);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
PARS_INST(kPathEscape, false)
PARS_INST(kPathEscape, true)
#undef PARS_INST

const void* scan_ws_batch_kernel(int path, bool brackets) {
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, false, true, 16>);
		case 1: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, true, true, 16>);
		case 2: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, false, true, 16>);
		case 3: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, true, true, 16>);
		case 4: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, false, true, 16>);
		case 5: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, true, true, 16>);
		case 6: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, false, true, 16>);
		case 7: return reinterpret_cast<const void*>(&k_scan_ws<kPathEscape, true, true, 16>);
		default: return nullptr;
	}
}

}  // namespace pars
