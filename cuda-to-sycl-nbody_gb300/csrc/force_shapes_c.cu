// Force kernel shapes 8-12: large j-tiles (1024 and 2048 particles, 48-96 KB of tile
// ring), which amortise the per-tile barrier, bulk-copy issue and Kahan step.
// 9 (256 x 4, 2048-particle tiles) is the default for large systems; 11 and 12
// (128 x 4, 512-particle i-tiles, two CTAs per SM) suit ensembles of uneven systems,
// whose i-tiles waste fewer lanes on padding.
#include "force_kernel.cuh"

namespace nbg {

extern const ConfigEntry kForceShapesC[] = {
    NBG_CONFIG(256, 4, 1024, 3, 4),
    NBG_CONFIG(256, 4, 2048, 3, 4),
    NBG_CONFIG(256, 2, 1024, 3, 4),
    NBG_CONFIG(128, 4, 1024, 3, 4),
    NBG_CONFIG(128, 4, 2048, 3, 4),
};
extern const int kNumForceShapesC = sizeof(kForceShapesC) / sizeof(kForceShapesC[0]);

}  // namespace nbg
