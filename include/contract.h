/*
 * contract.h -- drop-in C ABI of libcontract.so (GB300 build).
 *
 * Entry points, argument order and meaning are those of CLQCD/contract
 * include/contract.h:15-27; each declaration below names the reference
 * function it replaces.  Conventions shared by every call:
 *
 *  - Propagators are caller-owned DEVICE buffers of `volume` sites, each site
 *    144 complex128 values ordered [sink spin][source spin][sink colour]
 *    [source colour] (PyQUDA LatticePropagator order).
 *  - Correlators are caller-owned DEVICE buffers, one complex128 per site.
 *  - Gamma indices are 0..15 with Gamma(n) = g1^(n&1) g2^(n>>1&1) g3^(n>>2&1)
 *    g4^(n>>3&1) in the DeGrand-Rossi basis.
 *  - Work is queued on the library's current stream (the legacy default stream
 *    unless contract_set_stream() in contract_gb300.h changed it); calls return
 *    before the GPU finishes.  Nothing is allocated.
 *  - Invalid arguments are reported the way the reference reports them
 *    (message on stderr, then exit(-1)) unless contract_set_error_mode()
 *    selects recording; see contract_gb300.h.
 */
#ifndef CONTRACT_H
#define CONTRACT_H

#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#ifndef __cplusplus
#include <complex.h>
#endif

#include "contract_enum.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces init (lib/contract.cpp:65-68): makes `device` current for the calling thread. */
void init(int device);

/* Replaces meson_two_point (lib/contract.cpp:6-10, include/meson.cuh:33-76):
 * correl[x] = Tr[(g5 G_ij) S_i(x) (g5 G_kl) S_j(x)^dagger] over spin and colour. */
void meson_two_point(void *correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_ij, int gamma_kl);

/* Replaces meson_all_source_two_point (lib/contract.cpp:12-16, include/meson_all.cuh:53-80):
 * `correl` is a HOST array of 16 device pointers; correl[g] receives the
 * meson_two_point value with gamma_kl = g. */
void meson_all_source_two_point(void **correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_ij);

/* Replaces meson_all_sink_two_point (lib/contract.cpp:18-22, include/meson_all.cuh:83-111):
 * correl[g] receives the meson_two_point value with gamma_ij = g. */
void meson_all_sink_two_point(void **correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_kl);

/* Replaces baryon_diquark (lib/contract.cpp:24-28, include/diquark.cuh:33-84):
 * writes a propagator-shaped diquark field.  As in the reference, an invalid
 * gamma_ij makes the call a no-op. */
void baryon_diquark(void *diquark, void *propag_i, void *propag_j, size_t volume, int gamma_ij, int gamma_kl);

/* Replaces baryon_two_point (lib/contract.cpp:30-35, include/baryon.cuh:34-120). */
void baryon_two_point(void *correl, void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                      unsigned long volume, int gamma_ij, int gamma_kl, int gamma_mn);

/* Replaces baryon_general_two_point (lib/contract.cpp:37-44, include/baryon_general.cuh:36-127):
 * the Gamma_mn operand is the HOST array project_mn[16] (row-major 4x4). */
void baryon_general_two_point(void *correl, void *propag_i, void *propag_j, void *propag_n,
                              BaryonContractType contract_type, size_t volume, int gamma_ij, int gamma_kl,
#ifdef __cplusplus
                              void *project_mn
#else
                              double _Complex *project_mn
#endif
);

/* Replaces baryon_sequential_two_point (lib/contract.cpp:46-63, include/baryon_sequential.cuh):
 * overwrites the propagator selected by sequential_type with dC(x)/dP(x) of the
 * corresponding baryon_two_point; the other two are read only.  As in the
 * reference, an invalid sequential_type makes the call a no-op. */
void baryon_sequential_two_point(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                                 BaryonSequentialType sequential_type, size_t volume, int gamma_ij, int gamma_kl,
                                 int gamma_mn);

#ifdef __cplusplus
}
#endif

#endif /* CONTRACT_H */
