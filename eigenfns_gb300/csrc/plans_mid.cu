// FFT plans for the mid grid edges.
#include "plan.cuh"

namespace ef {

void add_plans_mid(std::vector<Plan>& v) {
  v.push_back(make_plan<8, 6>());   // G = 48
  v.push_back(make_plan<8, 8>());   // G = 64
  v.push_back(make_plan<12, 8>());   // G = 96
}

}  // namespace ef
