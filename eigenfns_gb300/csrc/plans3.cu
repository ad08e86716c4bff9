// Grid edges of the three-pass operator (zplane.cuh): x-classes Q, z-in split,
// sub-plane x and y splits, sub-planes per CTA and threads, z-out split.
#include "zplane.cuh"

namespace ef {

void add_plans3(std::vector<Plan3>& v) {
  //                 Q  z-in    x       y      PL  NT    z-out
  v.push_back(make_plan3<1, 4, 8, 4, 8, 4, 8, 4, 256, 8, 4>());         // G = 32
  v.push_back(make_plan3<1, 4, 12, 4, 12, 4, 12, 3, 192, 12, 4>());     // G = 48
  v.push_back(make_plan3<1, 8, 8, 8, 8, 8, 8, 2, 256, 8, 8>());         // G = 64
  v.push_back(make_plan3<1, 8, 12, 8, 12, 8, 12, 1, 384, 12, 8>());     // G = 96
  v.push_back(make_plan3<2, 8, 16, 8, 8, 8, 16, 1, 256, 16, 8>());      // G = 128
  v.push_back(make_plan3<4, 8, 24, 4, 12, 12, 16, 1, 256, 24, 8>());    // G = 192
  v.push_back(make_plan3<4, 8, 32, 8, 8, 16, 16, 1, 1024, 32, 8>());    // G = 256
}

}  // namespace ef
