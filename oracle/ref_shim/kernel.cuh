// Host-side stand-in for CLQCD/contract's include/kernel.cuh (test infrastructure only).
//
// oracle/Makefile puts this directory ahead of the reference's include/ on the
// include path, so the reference's op headers (meson.cuh, baryon.cuh, ...)
// compile as plain host C++ and their per-site *_local functions can be called
// from oracle/ref_*.cpp.  It supplies what those headers expect from
// kernel.cuh (kernel.cuh:28-45 colour-loop macros, kernel.cuh:55-151 ThreadTile,
// TileKernel), written for a CPU:
//
//  * ThreadTile<16> runs the 16 lanes of a tile as 16 host threads that meet
//    at a std::barrier; shfl/plus go through a shared scratch array.  Only the
//    sequential kernels need real lanes (baryon_sequential.cuh:87-88,110-111).
//  * atomicAdd(double*, double) is a std::atomic_ref fetch_add.
//
// The colour macros must enumerate the same (a,b,c,d,e,f) index sets and sum
// the same four epsilon-epsilon products in the same order as the reference,
// so that this host build reproduces the reference's arithmetic.
#pragma once

#include <atomic>
#include <barrier>
#include <cstddef>
#include <type_traits>

#include <kernel_define.cuh>
#include <complex.cuh>

#define shared_memory(_type, _name, _shape) _type _name _shape

// Cyclic colour triples: for a given first index a the other two are
// b = a+1, c = a+2 (mod 3); likewise (d, e, f).  `ad` is the flat (a, d) index.
#define for_a_d                                                                                        \
  for (int ad = 0, a = 0, d = 0; ad < 9; ++ad, a = ad / 3, d = ad % 3)

#define for_abc_def                                                                                    \
  for (int ad = 0, a = 0, d = 0, b = 1, c = 2, e = 1, f = 2; ad < 9;                                   \
       ++ad, a = ad / 3, d = ad % 3, b = (a + 1) % 3, c = (a + 2) % 3, e = (d + 1) % 3, f = (d + 2) % 3)

// sum_{bc,ef} eps_abc eps_def X[b,e] Y[c,f] for the current (a, d):
// (X_be Y_cf + X_cf Y_be) - (X_ce Y_bf + X_bf Y_ce).
#define epsilon_abc_def(_x, _y)                                                                        \
  ((_x[3 * b + e] * _y[3 * c + f] + _x[3 * c + f] * _y[3 * b + e]) -                                   \
   (_x[3 * c + e] * _y[3 * b + f] + _x[3 * b + f] * _y[3 * c + e]))

inline double atomicAdd(double *address, double value)
{
  return std::atomic_ref<double>(*address).fetch_add(value, std::memory_order_relaxed);
}

namespace contract
{
  // State shared by the 16 host threads that play one tile.
  struct HostTile {
    std::barrier<> bar{16};
    alignas(64) unsigned char slot[16][64];
  };

  template <unsigned int TILE_SIZE> struct ThreadTile {
    HostTile *host = nullptr;
    unsigned int lane = 0;

    unsigned int thread_rank() const { return lane; }
    unsigned int meta_group_rank() const { return 0; }
    void sync() const
    {
      if (host) host->bar.arrive_and_wait();
    }

    template <typename T> T shfl(T value, unsigned int src) const
    {
      static_assert(sizeof(T) <= 64, "slot too small");
      *reinterpret_cast<T *>(host->slot[lane]) = value;
      sync();
      T out = *reinterpret_cast<const T *>(host->slot[src]);
      sync();
      return out;
    }

    template <typename T> T shfl_down(T value, unsigned int delta) const
    {
      *reinterpret_cast<T *>(host->slot[lane]) = value;
      sync();
      T out = (lane + delta < TILE_SIZE) ? *reinterpret_cast<const T *>(host->slot[lane + delta]) : value;
      sync();
      return out;
    }

    // Every lane receives the lane-ordered sum (the device reduction only
    // guarantees it in lane 0; the callers broadcast from lane 0).
    template <unsigned int BLOCK_SIZE, typename T> T plus(T value) const
    {
      *reinterpret_cast<T *>(host->slot[lane]) = value;
      sync();
      T sum = *reinterpret_cast<const T *>(host->slot[0]);
      for (unsigned int l = 1; l < TILE_SIZE; ++l) sum += *reinterpret_cast<const T *>(host->slot[l]);
      sync();
      return sum;
    }
  };

  template <typename Args, unsigned int BLOCK_SIZE_, unsigned int TILE_SIZE_> struct BaseKernel {
    const Args &args;
    static constexpr unsigned int BLOCK_SIZE = BLOCK_SIZE_;
    static constexpr unsigned int TILE_SIZE = TILE_SIZE_;
    static constexpr unsigned int TILES_PER_BLOCK = BLOCK_SIZE_ / TILE_SIZE_;
    constexpr BaseKernel(const Args &a) : args(a) { }
  };

  template <typename Args, unsigned int BLOCK_SIZE_, unsigned int TILE_SIZE_>
  struct TileKernel : public BaseKernel<Args, BLOCK_SIZE_, TILE_SIZE_> {
    constexpr TileKernel(const Args &a) : BaseKernel<Args, BLOCK_SIZE_, TILE_SIZE_>(a) { }
    virtual void operator()(size_t x_offset, ThreadTile<TILE_SIZE_> tile) = 0;
  };
} // namespace contract
