// Strict build of the stream-collide kernels: compiled with -fmad=false and
// evaluated in the reference's expression order (update_ref), so binary32
// results equal the binary32 restatement of the WGSL kernels bit for bit.
#define PW_NS pwstrict
#define PW_STRICT 1
#define PW_DEFINE_LAUNCHERS
#include "pw_lbm.cuh"
#include "pw_lbm_tile.cuh"
