// Tile kernels (push + Esirkepov deposit + wrap) for 2D, shape order 1.
#include "tg_particles.cuh"

namespace tg {
template cudaError_t launch_tiles_o<2, 1>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
template cudaError_t launch_tail_o<2, 1>(const TileArgs &, const long long *, bool, cudaStream_t);
}  // namespace tg
