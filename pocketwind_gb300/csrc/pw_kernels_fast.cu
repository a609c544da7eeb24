// Fast build of the stream-collide kernels: fused multiply-add allowed and the
// hand-simplified moment algebra of update_fast().
#define PW_NS pwfast
#define PW_STRICT 0
#define PW_DEFINE_LAUNCHERS
#include "pw_lbm.cuh"

#include "pw_lbm_tile.cuh"
