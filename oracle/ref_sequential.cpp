// Host build of the reference's baryon_sequential_local
// (include/baryon_sequential.cuh:36-163).  That function needs real tile
// lanes (tile.sync, a tile all-reduce and shared-memory atomics), so each
// site is played by 16 host threads meeting at a barrier (ref_shim/kernel.cuh).
// The load/compute/store wiring of the three device kernels, including the
// i/j swap of the IM_* types, follows baryon_sequential.cuh:166-267.
#include <baryon_sequential.cuh>
#include "ref_common.h"

#include <cstring>
#include <thread>
#include <vector>

template <BaryonContractType CONTRACT, int GAMMA_MN, int SLOT>
static void run(cplx *gi, cplx *gj, cplx *gn, std::size_t volume, int gamma_ij, int gamma_kl)
{
  using T = contract::Complex<double>;
  constexpr bool swap_ij = (CONTRACT == IM_JK_NL || CONTRACT == IM_JL_NK);
  // (load buffers, computed local slot, stored buffer) per kernel
  constexpr BaryonSequentialType local_slot = SLOT == 2 ? SEQUENTIAL_N
    : (SLOT == 0 ? (swap_ij ? SEQUENTIAL_J : SEQUENTIAL_I) : (swap_ij ? SEQUENTIAL_I : SEQUENTIAL_J));

  contract::HostTile host;
  T si[16][9], sj[16][9], sn[16][9];

  auto load = [&](T (*dst)[9], const cplx *src) { std::memcpy(dst, src, sizeof(T) * kSite); };
  auto store = [&](cplx *dst, T (*src)[9]) { std::memcpy(dst, src, sizeof(T) * kSite); };

  auto lane_fn = [&](unsigned int lane) {
    contract::ThreadTile<16> tile;
    tile.host = &host;
    tile.lane = lane;
    for (std::size_t x = 0; x < volume; ++x) {
      if (lane == 0) {
        std::memset(si, 0, sizeof(si));
        std::memset(sj, 0, sizeof(sj));
        std::memset(sn, 0, sizeof(sn));
        const std::size_t o = x * kSite;
        if constexpr (SLOT == 0) {
          if constexpr (swap_ij) { load(si, gj + o); } else { load(sj, gj + o); }
          load(sn, gn + o);
        } else if constexpr (SLOT == 1) {
          if constexpr (swap_ij) { load(sj, gi + o); } else { load(si, gi + o); }
          load(sn, gn + o);
        } else {
          if constexpr (swap_ij) { load(si, gj + o); load(sj, gi + o); } else { load(si, gi + o); load(sj, gj + o); }
        }
      }
      tile.sync();
      contract::baryon_sequential_local<CONTRACT, local_slot, GAMMA_MN, double>(si, sj, sn, gamma_ij, gamma_kl,
                                                                               (int)lane, tile);
      tile.sync();
      if (lane == 0) {
        const std::size_t o = x * kSite;
        if constexpr (local_slot == SEQUENTIAL_I) store((SLOT == 0 ? gi : gj) + o, si);
        else if constexpr (local_slot == SEQUENTIAL_J) store((SLOT == 0 ? gi : gj) + o, sj);
        else store(gn + o, sn);
      }
      tile.sync();
    }
  };
  std::vector<std::thread> lanes;
  for (unsigned int l = 0; l < 16; ++l) lanes.emplace_back(lane_fn, l);
  for (auto &t : lanes) t.join();
}

extern "C" int ref_baryon_sequential_two_point(cplx *pi, cplx *pj, cplx *pn, int contract_type, int sequential_type,
                                               std::size_t volume, int gamma_ij, int gamma_kl, int gamma_mn)
{
  bool ok = false;
  dispatch_int<6>(contract_type, [&](auto c) {
    dispatch_int<16>(gamma_mn, [&](auto g) {
      ok = dispatch_int<3>(sequential_type, [&](auto s) {
        run<static_cast<BaryonContractType>(decltype(c)::value), decltype(g)::value, decltype(s)::value>(
          pi, pj, pn, volume, gamma_ij, gamma_kl);
      });
    });
  });
  return ok ? 0 : -1;
}
