// Kernel launchers of the x2dhf GB300 library (implemented in x2g_kernels.cu).
#pragma once

#include "x2g_internal.h"

namespace x2g {

constexpr int kMaxTerms = 36;  // orbitals in one Fock build (MAXORB)

// One term of the Fock potential of orbital iorb (src/fock.F90:102-160).
struct FockTerm {
  const double *coul;  // Coulomb potential of orbital iorb1 (ext)
  const double *ex;    // exchange potential K(iorb,iorb1) (ext), or null
  const double *ex2;   // second exchange potential (ilc2 == 2), or null
  const double *psi;   // orbital iorb1 (ext)
  double coo;          // occupation weight of the Coulomb term
  double gec, gec2;    // exchange weights (initExWeights)
  int mode;            // 0: iorb1 != iorb, 1: self term with m > 0 exchange, 2: self, no exchange
  int pad;
};

struct FockArgs {
  int nterms;
  int m;        // |lambda| of iorb
  int nel1;     // one-electron case: fockHF returns before the two-electron part
  int exact;    // 1: the reference's unfused FP64 order; 0 (mixed form): FMAs
  const double *ee;  // device: diagonal Lagrange multiplier of iorb
  double *lhs, *rhs; // plain outputs: fock1 + diag, fock2
  double *coulp, *exchp;  // plain: coulombptr, exchangeptr of iorb
  double *fa;        // 5 x nni: fock1/f1 on mu = nmu-5..nmu-1
  FockTerm t[kMaxTerms];
};

// Asymptotic boundary values (potAsympt, src/scfUtils.F90:179-329).
struct AsymptItem {
  double *pot;  // ext array
  int type;     // 0 Coulomb (cmulti of orbital `idx`), 1 exchange (moments slot `idx`)
  int idx;
  int idel;
  int pad;
};
constexpr int kMaxAsympt = 80;
struct AsymptArgs {
  int n;
  int norb;
  const double *cmulti;  // [norb][8] Coulomb moments
  const double *excm;    // [nslots][8] exchange moments
  int nslots;
  int pad;
  AsymptItem it[kMaxAsympt];
};

// ---- sweeps ----
int cluster_occupancy(x2g_ctx *ctx, x2g_grid *grid, int *plain, int *pot);
int launch_relax(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps, int precision);
// FP64 sweep whose job table, right-hand-side buffers and barrier words live
// in caller-provided device scratch (no allocation on this path).
size_t relax_scratch_bytes(const GridDev &g, int njobs);
int launch_relax_in_scratch(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps,
                            void *scratch, size_t scratch_bytes);

// ---- elementwise ----
void launch_ghost_fill(x2g_ctx *ctx, const GridDev &g, double *u, int isym);           // putin ghosts, all rows
void launch_putin(x2g_ctx *ctx, const GridDev &g, int isym, const double *plain, double *ext);
void launch_putout(x2g_ctx *ctx, const GridDev &g, const double *ext, double *plain);
void launch_fock(x2g_ctx *ctx, const GridDev &g, const FockArgs &a);
// Fock builds of n orbitals from the same state (a[0].exact for all)
void launch_fock_batch(x2g_ctx *ctx, const GridDev &g, const FockArgs *a, int n);
// per-orbital asymptotic decay of several orbitals (fa, edecay, psi by orbital)
struct OrbDecayList {
  const double *fa[kMaxTerms];
  double *edecay[kMaxTerms];
  double *psi[kMaxTerms];
};
void launch_asympt_get_batch(x2g_ctx *ctx, const GridDev &g, const OrbDecayList &L, int n);
void launch_asympt_set_batch(x2g_ctx *ctx, const GridDev &g, const OrbDecayList &L, int n);
void launch_asympt_get(x2g_ctx *ctx, const GridDev &g, const double *fa, double *edecay);
void launch_asympt_set(x2g_ctx *ctx, const GridDev &g, double *psi, const double *edecay);
void launch_setci(x2g_ctx *ctx, const GridDev &g, double *psi, int ihomo);
void launch_scale(x2g_ctx *ctx, const GridDev &g, double *psi, const double *norm_dev);
// psi /= sqrt(norm) then setCiOrb's symmetrisation, in one pass
void launch_scale_setci(x2g_ctx *ctx, const GridDev &g, double *psi, const double *norm_dev, int ihomo);
void launch_ortho_apply(x2g_ctx *ctx, const GridDev &g, double *psi, const double *const *others, int n,
                        const double *ovl_dev);
void launch_asympt(x2g_ctx *ctx, const GridDev &g, const AsymptArgs &a);
// narrow_f64 / widen_f32 against the hardware conversions on n values
int convert_selftest(x2g_ctx *ctx, long n, unsigned long long seed, unsigned long long *mismatches);
// fills g's exm (40 x mxsize) and asy (51 x 4 nni) tables; synchronous
int build_moment_tables(x2g_ctx *ctx, const GridDev &g, double *exm, double *asy);
void launch_zero(x2g_ctx *ctx, double *p, size_t n);

// ---- reductions (deterministic two-pass; results in device memory) ----
// norm: out[0] = sum wgt2 psi psi f4
void launch_norm(x2g_ctx *ctx, const GridDev &g, const double *psi, double *out);
// overlaps with n other orbitals: out[k] = sum wgt2 psi o_k f4
void launch_overlaps(x2g_ctx *ctx, const GridDev &g, const double *psi, const double *const *others, int n,
                     double *out);
// EaHF: out = woneel + (wcoul + wexch); psi must have ghosts filled.
// Also writes parts[0..4] = kinetic, nuclear, oneel, coul, exch.
// psi's ghost cells are read as mirrored interior values (no ghost refresh
// needed); exact: the reference's unfused FP64 order, else FMAs (mixed form)
void launch_eahf(x2g_ctx *ctx, const GridDev &g, const double *psi, int isym, int m, const double *coulp,
                 const double *exchp, double *ee_out, double *parts, bool exact = true);
// One orthonormalisation round over orbitals whose partners were finished
// in earlier rounds: norm (out norm_out), scaling by 1/sqrt(norm) (and
// setCiOrb with ihomo = +-1; 0 scales only), overlaps with the partners (out
// ovl_out) and the Gram-Schmidt step; the same sums and operations as
// launch_norm / launch_scale(_setci) / launch_overlaps / launch_ortho_apply.
struct OrthoOrbital {
  double *psi;
  const double *partners[16];
  int n, ihomo;
  double *norm_out, *ovl_out;
};
void launch_ortho_round(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, int n);
// all rounds in one cooperative launch (round r: orbs[round_off[r] ..
// round_off[r+1])); false: not launched, take launch_ortho_round per round
bool launch_orthonormalise(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, const int *round_off,
                           int nrounds);
// the same through the orbitals' inner products (one reduction pass, one
// grid barrier, one update pass), orbs in the reference's order with
// partner_index[j * 16 + p] the plan index of orbs[j].partners[p]; false:
// not launched
bool launch_orthonormalise_gram(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, int n,
                                const int *partner_index);
// EaHF of several orbitals in one launch (same sums, same order as launch_eahf)
struct EahfItem {
  const double *psi, *coulp, *exchp;
  double *ee_out, *parts;
  int isym, m;
};
void launch_eahf_batch(x2g_ctx *ctx, const GridDev &g, const EahfItem *items, int n, bool exact);
// generic weighted triple products: out[k] = sum w * a_k * b_k * c_k (c may be null), w = wgt2
struct TripleItem {
  const double *a, *b, *c;  // a,b ext arrays; c ext or null
};
void launch_triples(x2g_ctx *ctx, const GridDev &g, const TripleItem *items, int n, double *out);
// multipole moments
// a batch of moments, one launch per kMomentItems: coul != 0 is coulMom of
// psa (psb unused), else exchMom of the pair with idel
struct MomentItem {
  const double *psa, *psb;
  double *out;  // [mpole]
  int idel, coul;
};
void launch_moments(x2g_ctx *ctx, const GridDev &g, const MomentItem *items, int n, int homo);

}  // namespace x2g
