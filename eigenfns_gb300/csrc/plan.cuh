// FFT plan of one grid edge: the launchers of every pass kernel instantiated
// for its split G = R1 * R2. Plans are instantiated in plans_*.cu so the
// translation units compile in parallel.
#pragma once
#include <atomic>
#include <vector>

#include "fft_passes.cuh"
#include "status.h"

namespace ef {

using Launch = void (*)(dim3, size_t, cudaStream_t, const PassArgs&);

struct Plan {
  int G, R1, R2, NZ, PS;   // y/x passes: split R1 >= R2, NZ z-columns per tile
  int NRA, PSA;            // pass A: split (R2, R1), NRA rows per tile
  int NRE, PSE;            // pass E: split (R1, R2), NRE rows per tile
  Launch a[3];       // BuildMode
  Launch y[2];       // 0 inverse, 1 forward
  Launch c[4];       // WMode
  Launch e[8];       // EpiMode
};

template <class K>
void set_smem(K kernel, size_t smem) {
  set_smem_once(kernel, smem);
}

template <class GEO, int B>
void launch_a(dim3 g, size_t s, cudaStream_t st, const PassArgs& a) {
  set_smem(pass_a_kernel<GEO, B>, s);
  ef_count_launches(1);
  pass_a_kernel<GEO, B><<<g, kThreads, s, st>>>(a);
}
template <class GEO, int D>
void launch_y(dim3 g, size_t s, cudaStream_t st, const PassArgs& a) {
  set_smem(pass_y_kernel<GEO, D>, s);
  ef_count_launches(1);
  pass_y_kernel<GEO, D><<<g, kThreads, s, st>>>(a);
}
template <class GEO, int W>
void launch_c(dim3 g, size_t s, cudaStream_t st, const PassArgs& a) {
  set_smem(pass_c_kernel<GEO, W>, s);
  ef_count_launches(1);
  pass_c_kernel<GEO, W><<<g, kThreads, s, st>>>(a);
}
template <class GEO, int E>
void launch_e(dim3 g, size_t s, cudaStream_t st, const PassArgs& a) {
  set_smem(pass_e_kernel<GEO, E>, s);
  ef_count_launches(1);
  pass_e_kernel<GEO, E><<<g, kThreads, s, st>>>(a);
}

// y/x passes use the split (R1, R2); pass A uses (RA1, RA2) with the small factor
// first (the 3 components of RA1 voxels live in registers), pass E uses (RE1, RE2)
// with the small factor last (the 3 components of RE2 outputs live in registers).
template <int R1, int R2, int RA1 = R2, int RA2 = R1, int RE1 = R1, int RE2 = R2>
Plan make_plan() {
  using GY = Geo<R1, R2>;
  using GA = Geo<RA1, RA2>;
  using GE = Geo<RE1, RE2>;
  static_assert(GA::G == GY::G && GE::G == GY::G, "splits of one grid edge");
  Plan p;
  p.G = GY::G; p.R1 = R1; p.R2 = R2; p.NZ = GY::NZ; p.PS = GY::PS;
  p.NRA = GA::NRA; p.PSA = GA::PS;
  p.NRE = GE::NRE; p.PSE = GE::PS;
  p.a[0] = launch_a<GA, BUILD_THETA>;
  p.a[1] = launch_a<GA, BUILD_PRECOND>;
  p.a[2] = launch_a<GA, BUILD_CART>;
  p.y[0] = launch_y<GY, +1>;
  p.y[1] = launch_y<GY, -1>;
  p.c[0] = launch_c<GY, W_INV_EPS>;
  p.c[1] = launch_c<GY, W_EPS>;
  p.c[2] = launch_c<GY, W_INV_ONLY>;
  p.c[3] = launch_c<GY, W_INV_ONLY_EPS>;
  p.e[0] = launch_e<GE, EPI_THETA>;
  p.e[1] = launch_e<GE, EPI_PRECOND>;
  p.e[2] = launch_e<GE, EPI_CHEB>;
  p.e[3] = launch_e<GE, EPI_CHEB_FIRST>;
  p.e[4] = launch_e<GE, EPI_KPM>;
  p.e[5] = launch_e<GE, EPI_KPM_FIRST>;
  p.e[6] = launch_e<GE, EPI_KPM_COUNT>;
  p.e[7] = launch_e<GE, EPI_KPM_FIRST>;
  return p;
}

// each plans_*.cu appends its grid edges
void add_plans_small(std::vector<Plan>& v);
void add_plans_mid(std::vector<Plan>& v);
void add_plans_large(std::vector<Plan>& v);

}  // namespace ef
