// Force kernel shapes 0-3.  3 is the default for ensembles of small systems; 0 is the
// shape of nb_accelerations_noalloc.
#include "force_kernel.cuh"

namespace nbg {

extern const ConfigEntry kForceShapesA[] = {
    NBG_CONFIG(128, 4, 256, 3, 4),
    NBG_CONFIG(256, 4, 256, 3, 4),
    NBG_CONFIG(128, 8, 256, 3, 4),
    NBG_CONFIG(256, 2, 256, 3, 4),
};
extern const int kNumForceShapesA = sizeof(kForceShapesA) / sizeof(kForceShapesA[0]);

}  // namespace nbg
