/*
 * micsa_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the device path of IsidoroGlez/micSA-EA-MC
 * (PROGRAM/src/main.cu kernels and PROGRAM/src/med.c), operating on the
 * reference's own multispin-coded layout:
 *   spins   even/odd[h*nr + r]                (h_MSC_u_even/odd, ini.c:336)
 *   J       J[(p*6 + d)*H + h]                (d_J via viciniB/N, main.cu:443-455)
 *   demons  w[((p*nc + ic)*H + h)*nr + r]     (CPUwalker0/1, main.cu:355-362)
 * It is the checker for the CUDA path and the scalar CPU baseline; nothing
 * in the product links or calls it.
 *
 * Parity pin: tests compare it with the reference program itself, built for
 * the CPU from the reference sources (oracle/ref_cpu/build_ref.sh), and with
 * golden outputs of that build committed under tests/golden/.
 */
#ifndef MICSA_ORACLE_H
#define MICSA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* neighbour and rotate tables: neig[(p*6 + d)*H + h] = word index (other
 * colour) of the d-neighbour, rot[p*H + h] = bit d set when that neighbour
 * lies across a block edge (Init_MSC_index_and_rotate, ini.c:148-258). */
void oracle_tables(int L, int32_t *neig, uint8_t *rot);

/* one half-sweep of colour p on demon plane ic (d_oneMCstepBN_multisample,
 * main.cu:847-1080).  rand == NULL: microcanonical ISI update of demon
 * words w0/w1 (CPUwalker layout); rand != NULL: Metropolis with
 * rand[k*H*nr + h*nr + r], k = 0..2 (demons untouched).  Replicas r0..r1-1. */
void oracle_half_sweep(int L, int nr, int nc, int p, int ic, const uint64_t *J,
                       uint64_t *even, uint64_t *odd, uint64_t *w0,
                       uint64_t *w1, const uint64_t *rand, int r0, int r1);

/* demon walk, both colours (d_Walk dir 0 then 1, main.cu:285-305,1084-1193) */
void oracle_walk(int L, int nr, int nc, uint64_t *w0, uint64_t *w1, int r0,
                 int r1);

/* one micSA iteration: nc x (even, odd) sweeps then the walk (Monte_Carlo
 * flag=1, main.cu:254-305), split over `nthreads` threads by replica. */
void oracle_micsa_iteration(int L, int nr, int nc, const uint64_t *J,
                            uint64_t *even, uint64_t *odd, uint64_t *w0,
                            uint64_t *w1, int nthreads);

/* Philox4x32-10 + LUT bisection random words (d_gen_rndbits_cuda,
 * main.cu:546-702): te[r*4+k] counters, keys[r], lut = 4096-byte
 * s_lut_heat_bath; out[k*H*nr + h*nr + r], k = 0..2. */
void oracle_gen_rndbits(int L, int nr, const uint32_t *te, const uint32_t *keys,
                        const void *lut, uint64_t *out);

/* Metropolis iteration (Monte_Carlo flag=0, main.cu:206-253) given the
 * counters of the even (te0) and odd (te1) calls. */
void oracle_metropolis_iteration(int L, int nr, const uint64_t *J,
                                 uint64_t *even, uint64_t *odd,
                                 const uint32_t *te0, const uint32_t *te1,
                                 const uint32_t *keys, const void *lut);

/* spin energy per replica, h_Ener = 3V - 2 * unsatisfied bonds
 * (d_computeEne, main.cu:745-815) */
void oracle_energy(int L, int nr, const uint64_t *J, const uint64_t *even,
                   const uint64_t *odd, int32_t *ener);

/* demon energy per replica (Measure_Energy_Clerics, med.c:55-83) */
void oracle_demon_energy(int L, int nr, int nc, const uint64_t *w0,
                         const uint64_t *w1, uint64_t *ener);

/* the ISI demon algebra on one word (main.cu:1037-1074) */
uint64_t oracle_isi_word(uint64_t j1, uint64_t j2, uint64_t j3, uint64_t j4,
                         uint64_t *D0, uint64_t *D1);

/* coupling words J[(p*6 + d)*H + h] from per-site couplings J{x,y,z}[x +
 * L*y + L*L*z] in {0,1} (packing_J, ini.c:521-578) */
void oracle_pack_couplings(int L, const uint8_t *Jx, const uint8_t *Jy,
                           const uint8_t *Jz, uint64_t *J);

/* ---- plain scalar rendering on unpacked spins uu[r*V + x+L*y+L*L*z] ---- */
/* accept/demon rule per site: returns new demon, sets *flip */
int oracle_scalar_rule(int unsatisfied, int demon, int *flip);
/* overlap of pairs (2k, 2k+1): q[k] = sum_x s^a_x s^b_x, and
 * c4[(k*3 + axis)*(L/2+1) + d] = sum_x q_x q_{x+d e_axis}, d = 0..L/2 */
void oracle_overlap_c4(int L, int nr, const uint8_t *uu, int64_t *q,
                       int64_t *c4);
/* energy from unpacked spins (calculate_scalar_energy, med.c:85-114) */
int32_t oracle_scalar_energy(int L, const uint8_t *u, const uint8_t *Jx,
                             const uint8_t *Jy, const uint8_t *Jz);

#ifdef __cplusplus
}
#endif
#endif
