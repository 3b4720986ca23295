// Force kernel shapes 4-7 (small j-tiles for small systems; larger i-blocks).
#include "force_kernel.cuh"

namespace nbg {

extern const ConfigEntry kForceShapesB[] = {
    NBG_CONFIG(128, 2, 128, 3, 4),
    NBG_CONFIG(64, 4, 128, 3, 4),
    NBG_CONFIG(128, 6, 256, 3, 4),
    NBG_CONFIG(64, 8, 256, 3, 4),
};
extern const int kNumForceShapesB = sizeof(kForceShapesB) / sizeof(kForceShapesB[0]);

}  // namespace nbg
