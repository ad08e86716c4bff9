// FFT plans for the small grid edges.
#include "plan.cuh"

namespace ef {

void add_plans_small(std::vector<Plan>& v) {
  v.push_back(make_plan<4, 1>());   // G = 4
  v.push_back(make_plan<6, 1>());   // G = 6
  v.push_back(make_plan<8, 1>());   // G = 8
  v.push_back(make_plan<12, 1>());   // G = 12
  v.push_back(make_plan<16, 1>());   // G = 16
  v.push_back(make_plan<8, 3>());   // G = 24
  v.push_back(make_plan<8, 4>());   // G = 32
}

}  // namespace ef
