// FFT plans for the large grid edges.
#include "plan.cuh"

namespace ef {

void add_plans_large(std::vector<Plan>& v) {
  v.push_back(make_plan<16, 8>());   // G = 128
  v.push_back(make_plan<16, 12, 8, 24, 24, 8>());   // G = 192
  v.push_back(make_plan<16, 16, 8, 32, 32, 8>());   // G = 256
}

}  // namespace ef
