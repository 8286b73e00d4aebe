// Tile kernels (push + Esirkepov deposit + wrap) for 3D, shape order 3.
#include "tg_particles.cuh"

namespace tg {
template cudaError_t launch_tiles_o<3, 3>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
}  // namespace tg
