// Grid edges of the three-pass operator (zplane.cuh): z-in split, plane split with
// planes per CTA and threads, z-out split.
#include "zplane.cuh"

namespace ef {

void add_plans3(std::vector<Plan3>& v) {
  v.push_back(make_plan3<4, 8, 4, 8, 4, 256, 8, 4>());       // G = 32
  v.push_back(make_plan3<4, 12, 4, 12, 3, 192, 12, 4>());    // G = 48
  v.push_back(make_plan3<8, 8, 8, 8, 2, 256, 8, 8>());       // G = 64
  v.push_back(make_plan3<8, 12, 8, 12, 1, 384, 12, 8>());    // G = 96
  v.push_back(make_plan3<8, 16, 8, 16, 1, 1024, 16, 8>());    // G = 128
}

}  // namespace ef
