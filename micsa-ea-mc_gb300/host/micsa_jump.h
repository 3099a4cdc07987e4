/*
 * Jump-ahead of the demon-refresh generators, so that the draws of one
 * refresh (InitWalkers, ini.c:712-781) can be produced by many GPU threads,
 * each starting at its own offset, with exactly the reference's values.
 *
 * The three generators are linear:
 *   congruential  z -> A z + 1 (mod 2^64): o steps are one affine map;
 *   lagged Fibonacci x_k = x_{k-24} + x_{k-55} (mod 2^64): x_{m} for any m
 *     is a combination of a 55-value window, with coefficients
 *     X^t mod (X^55 - X^31 - 1);
 *   xoshiro256 state (GF(2)-linear): T^o = q(T) with q = X^o mod p, p the
 *     characteristic polynomial of T (degree 256).
 */
#ifndef MICSA_JUMP_H
#define MICSA_JUMP_H

#include <stdint.h>

#include "micsa_host.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MICSA_FIB_R 55 /* order of the lagged Fibonacci recurrence */

/* z_o = mult * z_0 + add after o congruential steps */
void micsa_lcg_jump(uint64_t o, uint64_t *mult, uint64_t *add);
/* coefficients c[0..54] of X^t mod (X^55 - X^31 - 1) over Z/2^64 */
void micsa_fib_jump(uint64_t t, uint64_t c[MICSA_FIB_R]);
/* 257-bit characteristic polynomial of the xoshiro256 transition
 * (bit i of p[i/64]; p[4] holds bit 256) */
void micsa_xoshiro_charpoly(uint64_t p[5]);
/* q = X^o mod p (256 bits) */
void micsa_xoshiro_jump_poly(uint64_t o, uint64_t q[4]);
/* s <- T^o s using q = X^o mod p */
void micsa_xoshiro_apply(const uint64_t q[4], uint64_t s[4]);

/* Advance one PR+congruential / xoshiro stream pair by n draws, leaving both
 * structs exactly as n calls of the sequential update would (every field). */
void micsa_streams_advance(micsa_prc_t *prc, micsa_xoshiro_t *xo, uint64_t n);

/* Per-segment jump tables of one refresh shape: segment g covers draws
 * [g*S, min((g+1)*S, M)), S = 64*words_per_seg, M = 64*nwords.
 *   lcg[2g], lcg[2g+1]   congruential map to the state before draw g*S
 *   xo[4g..4g+3]         X^(g*S) mod p
 *   fib[55g..55g+54]     X^(g*S - 6) mod (X^55 - X^31 - 1), g >= 1: the
 *                        window x_{gS-61} .. x_{gS-7} is
 *                        x_{gS-61+j} = sum_i fib[i] * E[i+j], E below.
 * and the jump of the whole refresh, for the host's own copy of the streams:
 *   adv_lcg (M-1 steps), adv_xo = X^(M-1) mod p, adv_fib = X^(M-202).     */
typedef struct {
  int64_t nwords, words_per_seg, nseg;
  uint64_t *lcg, *xo, *fib;
  uint64_t adv_lcg[2], adv_xo[4], adv_fib[MICSA_FIB_R];
} micsa_refresh_plan;
int micsa_refresh_plan_make(int64_t nwords, int64_t words_per_seg, micsa_refresh_plan *plan);
void micsa_refresh_plan_free(micsa_refresh_plan *plan);

/* Compact start state of one stream for the segmented generator:
 *   rec[0..5]     x_{-61} .. x_{-56}   (output lag only)
 *   rec[6..114]   E[k] = x_{-55+k}, k = 0..108 (the 55-value window and
 *                 54 further values of the recurrence)
 *   rec[115]      congruential state;  rec[116..119] xoshiro state.
 * Returns -1 if the ring pointers do not have the lags 24, 55, 61. */
#define MICSA_STREAM_REC 120
int micsa_stream_record(const micsa_prc_t *prc, const micsa_xoshiro_t *xo,
                        uint64_t rec[MICSA_STREAM_REC]);
/* Advance both structs by the plan's M draws (same result as M steps). */
void micsa_streams_advance_plan(const micsa_refresh_plan *plan, micsa_prc_t *prc,
                                micsa_xoshiro_t *xo);

/* CPU rendering of the segmented generation a GPU warp lane performs: draws
 * segment g of one stream from its record into w0/w1[i*nr + r] for the
 * segment's words; used to test the tables. */
void micsa_draw_segment(const micsa_refresh_plan *plan, int64_t g,
                        const uint64_t rec[MICSA_STREAM_REC], const uint64_t thr[3], int nr,
                        int r, uint64_t *w0, uint64_t *w1);

#ifdef __cplusplus
}
#endif
#endif
