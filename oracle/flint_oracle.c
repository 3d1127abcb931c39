/*
 * flint_oracle.c -- FP64 CPU oracle of FLINT's per-cell chemistry path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU library and the timed CPU
 * baseline.  Nothing in the product path links or calls it.
 *
 * What follows the reference line by line (paths within the FLINT project):
 *   - table lerp a+(b-a)*Tdiff            src/lib/Lib_Chemistry_data.f90:36-61,
 *                                         src/lib/Lib_ThermoTransport.f90:516-542
 *   - general loop                         src/lib/Lib_Chemistry_wdot.f90:96-220
 *   - Lindemann / Troe blending, f_F       src/lib/Lib_Chemistry_falloff.f90:12-80
 *   - rhs_native (constant volume)         src/lib/Lib_Chemistry_rhs.f90:15-52
 * What is new math written from the formulae FLINT's tables were generated with
 * (docs/theory_kinetics.md, docs/input_yaml.md:176-209; Cantera's conventions,
 * pinned by the golden tables):
 *   - NASA-7 cp/h/s, Kc = exp(-dG/RT) (p_ref/RT)^dnu, Troe Fcent(T)
 *   - the analytic Jacobian of the constant-pressure reactor
 *   - the BDF/Newton reactor (OSlo, the reference's integrator, is absent).
 *
 * Built with -ffp-contract=off so that every product and sum is rounded as
 * written.
 */
#include "flint_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXNS 128

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ------------------------------------------------------------------ thermo */
/* NASA-9: cp/R = a1/T^2 + a2/T + a3 + a4 T + a5 T^2 + a6 T^3 + a7 T^4,
 * h/RT = -a1/T^2 + a2 ln(T)/T + a3 + a4 T/2 + ... + a7 T^4/5 + b1/T,
 * s/R = -a1/(2 T^2) - a2/T + a3 ln T + a4 T + ... + a7 T^4/4 + b2. */
static void nasa9_thermo(const double* c, double T, double lnT, double* cpR, double* hRT, double* sR,
                         double* dcpR) {
  int nr = (int)c[0], r = 0;
  if (nr > 1 && T > c[2]) r = 1;
  if (nr > 2 && T > c[3]) r = 2;
  const double* a = c + 5 + 9 * r;
  double T2 = T * T, T3 = T2 * T, T4 = T3 * T, iT = 1.0 / T, iT2 = iT * iT;
  if (cpR) cpR[0] = a[0] * iT2 + a[1] * iT + a[2] + a[3] * T + a[4] * T2 + a[5] * T3 + a[6] * T4;
  if (hRT) hRT[0] = -a[0] * iT2 + a[1] * lnT * iT + a[2] + a[3] * T / 2.0 + a[4] * T2 / 3.0 + a[5] * T3 / 4.0
                    + a[6] * T4 / 5.0 + a[7] * iT;
  if (sR) sR[0] = -a[0] * iT2 / 2.0 - a[1] * iT + a[2] * lnT + a[3] * T + a[4] * T2 / 2.0 + a[5] * T3 / 3.0
                  + a[6] * T4 / 4.0 + a[8];
  if (dcpR) dcpR[0] = -2.0 * a[0] * iT2 * iT - a[1] * iT2 + a[3] + 2.0 * a[4] * T + 3.0 * a[5] * T2 + 4.0 * a[6] * T3;
}

void orc_species_thermo(const flint_mech_desc* m, double T, double* cpR, double* hRT,
                        double* sR, double* dcpR) {
  double lnT = log(T);
  if (m->nasa9) {
    for (int k = 0; k < m->ns; ++k)
      nasa9_thermo(m->nasa9 + 32 * k, T, lnT, cpR ? cpR + k : NULL, hRT ? hRT + k : NULL, sR ? sR + k : NULL,
                   dcpR ? dcpR + k : NULL);
    return;
  }
  for (int k = 0; k < m->ns; ++k) {
    const double* c = m->nasa7 + 17 * k;
    const double* a = (T <= c[1]) ? c + 3 : c + 10;
    double T2 = T * T, T3 = T2 * T, T4 = T3 * T;
    if (cpR) cpR[k] = a[0] + a[1] * T + a[2] * T2 + a[3] * T3 + a[4] * T4;
    if (hRT) hRT[k] = a[0] + a[1] * T / 2.0 + a[2] * T2 / 3.0 + a[3] * T3 / 4.0 + a[4] * T4 / 5.0 + a[5] / T;
    if (sR) sR[k] = a[0] * lnT + a[1] * T + a[2] * T2 / 2.0 + a[3] * T3 / 3.0 + a[4] * T4 / 4.0 + a[6];
    if (dcpR) dcpR[k] = a[1] + 2.0 * a[2] * T + 3.0 * a[3] * T2 + 4.0 * a[4] * T3;
  }
}

static double troe_fcent(const double* tr, double T, double* dFc) {
  double a = tr[0], T3 = tr[1], T1 = tr[2], T2 = tr[3];
  double e3 = exp(-T / T3), e1 = exp(-T / T1);
  double Fc = (1.0 - a) * e3 + a * e1;
  double d = -(1.0 - a) / T3 * e3 - a / T1 * e1;
  if (T2 != 0.0) {
    double e2 = exp(-T2 / T);
    Fc += e2;
    d += T2 / (T * T) * e2;
  }
  if (dFc) *dFc = d;
  return Fc;
}

/* ln Kc and d ln Kc / dT of reaction r. */
static void lnkc(const flint_mech_desc* m, int r, double T, const double* gRT, const double* hRT,
                 double* lk, double* dlk) {
  double dG = 0.0, dH = 0.0, dnu = 0.0;
  for (int s = 0; s < FLINT_MAXSP_PER_SIDE; ++s) {
    int sp = m->psp[3 * r + s];
    if (sp >= 0) {
      double nu = m->pnu[3 * r + s];
      dG += nu * gRT[sp]; dH += nu * hRT[sp]; dnu += nu;
    }
    sp = m->rsp[3 * r + s];
    if (sp >= 0) {
      double nu = m->rnu[3 * r + s];
      dG -= nu * gRT[sp]; dH -= nu * hRT[sp]; dnu -= nu;
    }
  }
  *lk = -dG + dnu * log(m->p_ref / (m->r_thermo * T));
  *dlk = (dH - dnu) / T;
}

void orc_rate_constants(const flint_mech_desc* m, double T, double* kf, double* Kc,
                        double* k0, double* fcent) {
  int ns = m->ns;
  double cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS];
  orc_species_thermo(m, T, cpR, hRT, sR, NULL);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  double lnT = log(T);
  for (int r = 0; r < m->nr; ++r) {
    const double* ar = m->arrh + 3 * r;
    if (kf) kf[r] = ar[0] * exp(ar[1] * lnT - ar[2] / T);
    int t = m->rtype[r];
    if (k0) {
      const double* a0 = m->arrh0 + 3 * r;
      k0[r] = (t >= FLINT_RXN_LINDEMANN) ? a0[0] * exp(a0[1] * lnT - a0[2] / T) : 0.0;
    }
    if (fcent) fcent[r] = (t == FLINT_RXN_TROE) ? troe_fcent(m->troe + 4 * r, T, NULL) : 1.0;
    if (Kc) {
      double lk, dlk;
      lnkc(m, r, T, gRT, hRT, &lk, &dlk);
      Kc[r] = m->reversible[r] ? exp(lk) : 0.0;
    }
  }
}

/* c^ord with its derivative.  Integral orders 0..4 use repeated products
 * (as coi**nint(ni) in the general loop, Lib_Chemistry_wdot.f90:140-141);
 * non-integral orders use pow on max(c,0). */
static void powd(double c, double ord, double* pw, double* dpw) {
  double fo = floor(ord);
  if (fo == ord && ord >= 0.0 && ord <= 4.0) {
    int n = (int)ord;
    if (n == 0) { *pw = 1.0; *dpw = 0.0; return; }
    double p = 1.0;
    for (int i = 0; i < n - 1; ++i) p *= c;
    *dpw = (double)n * p;
    *pw = p * c;
    return;
  }
  double cc = c > 0.0 ? c : 0.0;
  *pw = pow(cc, ord);
  *dpw = cc > 0.0 ? ord * pow(cc, ord - 1.0) : 0.0;
}

/* Kinetics of one cell in concentration space.
 * wm[k]   = sum_r nu_kr q_r            (molar, kmol/m^3/s)
 * wabs[k] = sum_r |nu_kr| (|fwd|+|rev|)
 * Jc[j*ns+k] = d wm_k / d c_j  (column j), Jcabs its absolute scale
 * JT[k]   = d wm_k / dT at fixed c, JTabs its scale.
 * Jc/JT may be NULL. */
static void kinetics(const flint_mech_desc* m, double T, const double* c,
                     const double* hRT, const double* gRT,
                     double* wm, double* wabs, double* Jc, double* Jcabs, double* JT, double* JTabs) {
  int ns = m->ns;
  double lnT = log(T), invT = 1.0 / T;
  for (int k = 0; k < ns; ++k) { wm[k] = 0.0; wabs[k] = 0.0; }
  if (Jc) {
    memset(Jc, 0, sizeof(double) * ns * ns);
    memset(Jcabs, 0, sizeof(double) * ns * ns);
    memset(JT, 0, sizeof(double) * ns);
    memset(JTabs, 0, sizeof(double) * ns);
  }
  double dqdc[MAXNS], dqabs[MAXNS];
  for (int r = 0; r < m->nr; ++r) {
    const double* ar = m->arrh + 3 * r;
    int type = m->rtype[r];
    double kf = ar[0] * exp(ar[1] * lnT - ar[2] * invT);
    double dlnkf = (ar[1] + ar[2] * invT) * invT;
    /* forward product */
    double pwf[3], dpwf[3], pwr[3], dpwr[3];
    int spf[3], spr[3];
    double Pf = 1.0, Pr = 1.0;
    for (int s = 0; s < 3; ++s) {
      spf[s] = m->rsp[3 * r + s];
      if (spf[s] >= 0) powd(c[spf[s]], m->rord[3 * r + s], &pwf[s], &dpwf[s]);
      else { pwf[s] = 1.0; dpwf[s] = 0.0; }
      Pf *= pwf[s];
    }
    int rev = m->reversible[r];
    double Kc = 0.0, dlnKc = 0.0, invKc = 0.0;
    if (rev) {
      double lk;
      lnkc(m, r, T, gRT, hRT, &lk, &dlnKc);
      invKc = exp(-lk);
      Kc = 1.0 / invKc;
      for (int s = 0; s < 3; ++s) {
        spr[s] = m->psp[3 * r + s];
        if (spr[s] >= 0) powd(c[spr[s]], m->pnu[3 * r + s], &pwr[s], &dpwr[s]);
        else { pwr[s] = 1.0; dpwr[s] = 0.0; }
        Pr *= pwr[s];
      }
    } else {
      Pr = 0.0;
      for (int s = 0; s < 3; ++s) { spr[s] = -1; pwr[s] = 1.0; dpwr[s] = 0.0; }
    }
    (void)Kc;
    /* third-body concentration */
    double M = 1.0, Mabs = 1.0;
    const double* eff = m->eff + (size_t)r * ns;
    if (type != FLINT_RXN_ELEMENTARY) {
      M = 0.0; Mabs = 0.0;
      for (int k = 0; k < ns; ++k) { M += eff[k] * c[k]; Mabs += fabs(eff[k] * c[k]); }
    }
    /* effective forward coefficient, its log-T derivative and its M-derivative */
    double keff, dlnkeff, dkeff_dM = 0.0, Mfac;  /* q = Mfac*keff*(Pf - Pr/Kc) */
    if (type == FLINT_RXN_ELEMENTARY) {
      keff = kf; dlnkeff = dlnkf; Mfac = 1.0;
    } else if (type == FLINT_RXN_THREEBODY) {
      keff = kf; dlnkeff = dlnkf; Mfac = M;
    } else {
      const double* a0 = m->arrh0 + 3 * r;
      double k0 = a0[0] * exp(a0[1] * lnT - a0[2] * invT);
      double dlnk0 = (a0[1] + a0[2] * invT) * invT;
      double kratio = k0 / kf;
      double Prd = kratio * M;
      double F = 1.0, G = 0.0, dlnF_T_Pr = 0.0;
      if (type == FLINT_RXN_TROE) {
        double dFc;
        double Fc = troe_fcent(m->troe + 4 * r, T, &dFc);
        double logFc = log10(Fc);
        double cc = -0.4 - 0.67 * logFc;
        double nn = 0.75 - 1.27 * logFc;
        double lPr = log10(Prd > 1e-300 ? Prd : 1e-300);
        double x = lPr + cc;
        double den = nn - 0.14 * x;
        double f1 = x / den;
        double opf = 1.0 + f1 * f1;
        F = pow(10.0, logFc / opf);
        double Aq = 2.0 * logFc * f1 / (opf * opf * den * den);
        G = -Aq * nn;
        dlnF_T_Pr = (1.0 / opf + Aq * (0.67 * nn - 1.27 * x)) * dFc / Fc;
      }
      double opr = 1.0 + Prd;
      keff = kf * (Prd / opr) * F;
      double dlnPr = dlnk0 - dlnkf;
      dlnkeff = dlnkf + dlnPr / opr + G * dlnPr + dlnF_T_Pr;
      /* d keff / d M = kinf * F/(1+Pr) * (1/(1+Pr) + G) * kratio */
      dkeff_dM = kf * F / opr * (1.0 / opr + G) * kratio;
      Mfac = 1.0;
    }
    double fwd = Mfac * keff * Pf;
    double rvs = rev ? Mfac * keff * invKc * Pr : 0.0;
    double q = fwd - rvs;
    double qabs = fabs(fwd) + fabs(rvs);
    /* species production */
    for (int s = 0; s < 3; ++s) {
      if (spf[s] >= 0) { wm[spf[s]] -= m->rnu[3 * r + s] * q; wabs[spf[s]] += fabs(m->rnu[3 * r + s]) * qabs; }
      int sp = m->psp[3 * r + s];
      if (sp >= 0) { wm[sp] += m->pnu[3 * r + s] * q; wabs[sp] += fabs(m->pnu[3 * r + s]) * qabs; }
    }
    if (!Jc) continue;
    /* dq/dc_j */
    for (int k = 0; k < ns; ++k) { dqdc[k] = 0.0; dqabs[k] = 0.0; }
    for (int s = 0; s < 3; ++s) {
      if (spf[s] >= 0) {
        double d = dpwf[s];
        for (int u = 0; u < 3; ++u) if (u != s) d *= pwf[u];
        double t = Mfac * keff * d;
        dqdc[spf[s]] += t; dqabs[spf[s]] += fabs(t);
      }
      if (rev && spr[s] >= 0) {
        double d = dpwr[s];
        for (int u = 0; u < 3; ++u) if (u != s) d *= pwr[u];
        double t = Mfac * keff * invKc * d;
        dqdc[spr[s]] -= t; dqabs[spr[s]] += fabs(t);
      }
    }
    if (type == FLINT_RXN_THREEBODY) {
      double base = keff * (Pf - (rev ? invKc * Pr : 0.0));
      double babs = fabs(keff * Pf) + (rev ? fabs(keff * invKc * Pr) : 0.0);
      for (int k = 0; k < ns; ++k) { dqdc[k] += eff[k] * base; dqabs[k] += fabs(eff[k]) * babs; }
    } else if (type >= FLINT_RXN_LINDEMANN) {
      double base = dkeff_dM * (Pf - (rev ? invKc * Pr : 0.0));
      double babs = fabs(dkeff_dM) * (fabs(Pf) + (rev ? fabs(invKc * Pr) : 0.0));
      for (int k = 0; k < ns; ++k) { dqdc[k] += eff[k] * base; dqabs[k] += fabs(eff[k]) * babs; }
    }
    /* dq/dT at fixed c */
    double dqT = fwd * dlnkeff - rvs * (dlnkeff - dlnKc);
    double dqTabs = fabs(fwd * dlnkeff) + fabs(rvs) * (fabs(dlnkeff) + fabs(dlnKc));
    for (int s = 0; s < 3; ++s) {
      int sps[2] = {spf[s], m->psp[3 * r + s]};
      double nus[2] = {-m->rnu[3 * r + s], m->pnu[3 * r + s]};
      for (int side = 0; side < 2; ++side) {
        int k = sps[side];
        if (k < 0) continue;
        double nu = nus[side];
        for (int j = 0; j < ns; ++j) {
          Jc[j * ns + k] += nu * dqdc[j];
          Jcabs[j * ns + k] += fabs(nu) * dqabs[j];
        }
        JT[k] += nu * dqT;
        JTabs[k] += fabs(nu) * dqTabs;
      }
    }
  }
}

static void cell_state(const flint_mech_desc* m, double T, double p, const double* Y,
                       double* c, double* rho_out, double* wbar_out) {
  int ns = m->ns;
  double sumYW = 0.0;
  for (int k = 0; k < ns; ++k) sumYW += Y[k] / m->mw[k];
  double rho = p / (m->r_eos * T * sumYW);
  for (int k = 0; k < ns; ++k) c[k] = rho * Y[k] / m->mw[k];
  if (rho_out) *rho_out = rho;
  if (wbar_out) *wbar_out = 1.0 / sumYW;
}

void orc_wdot_cell(const flint_mech_desc* m, double T, double p, const double* Y,
                   double* wdot, double* wscale, double* cp, double* h) {
  int ns = m->ns;
  double c[MAXNS], cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS], wm[MAXNS], wabs[MAXNS];
  cell_state(m, T, p, Y, c, NULL, NULL);
  orc_species_thermo(m, T, cpR, hRT, sR, NULL);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  kinetics(m, T, c, hRT, gRT, wm, wabs, NULL, NULL, NULL, NULL);
  for (int k = 0; k < ns; ++k) {
    if (wdot) wdot[k] = m->mw[k] * wm[k];
    if (wscale) wscale[k] = m->mw[k] * wabs[k];
  }
  if (cp || h) {
    double cps = 0.0, hs = 0.0;
    for (int k = 0; k < ns; ++k) {
      cps += Y[k] * cpR[k] / m->mw[k];
      hs += Y[k] * hRT[k] / m->mw[k];
    }
    if (cp) *cp = cps * m->r_thermo;
    if (h) *h = hs * m->r_thermo * T;
  }
}

void orc_rhs_constp_cell(const flint_mech_desc* m, double T, double p, const double* Y, double* f) {
  int ns = m->ns;
  double c[MAXNS], cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS], wm[MAXNS], wabs[MAXNS], rho;
  cell_state(m, T, p, Y, c, &rho, NULL);
  orc_species_thermo(m, T, cpR, hRT, sR, NULL);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  kinetics(m, T, c, hRT, gRT, wm, wabs, NULL, NULL, NULL, NULL);
  double Q = 0.0, D = 0.0;
  for (int k = 0; k < ns; ++k) {
    f[k] = m->mw[k] * wm[k] / rho;
    Q += hRT[k] * wm[k];
    D += c[k] * cpR[k];
  }
  f[ns] = -T * Q / D;
}

void orc_jac_cell(const flint_mech_desc* m, double T, double p, const double* Y,
                  double* f, double* J, double* Js) {
  int ns = m->ns, n = ns + 1;
  double c[MAXNS], cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS], dcpR[MAXNS];
  double wm[MAXNS], wabs[MAXNS], JT[MAXNS], JTa[MAXNS], S[MAXNS], Sa[MAXNS];
  double* Jc = (double*)malloc(sizeof(double) * ns * ns * 2);
  double* Jca = Jc + ns * ns;
  double rho, wbar;
  cell_state(m, T, p, Y, c, &rho, &wbar);
  orc_species_thermo(m, T, cpR, hRT, sR, dcpR);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  kinetics(m, T, c, hRT, gRT, wm, wabs, Jc, Jca, JT, JTa);
  double Q = 0.0, Qa = 0.0, D = 0.0;
  for (int k = 0; k < ns; ++k) {
    S[k] = 0.0; Sa[k] = 0.0;
    for (int j = 0; j < ns; ++j) {
      S[k] += c[j] * Jc[j * ns + k];
      Sa[k] += fabs(c[j]) * Jca[j * ns + k];
    }
    Q += hRT[k] * wm[k];
    Qa += fabs(hRT[k]) * wabs[k];
    D += c[k] * cpR[k];
  }
  for (int k = 0; k < ns; ++k) f[k] = m->mw[k] * wm[k] / rho;
  f[ns] = -T * Q / D;
  double wr = wbar / rho;
  /* species rows */
  for (int k = 0; k < ns; ++k) {
    double tk = S[k] - wm[k];
    double tka = Sa[k] + wabs[k];
    for (int mm = 0; mm < ns; ++mm) {
      double ratio = m->mw[k] / m->mw[mm];
      J[mm * n + k] = ratio * (Jc[mm * ns + k] - wr * tk);
      if (Js) Js[mm * n + k] = ratio * (Jca[mm * ns + k] + wr * tka);
    }
    J[ns * n + k] = (m->mw[k] / rho) * (JT[k] - tk / T);
    if (Js) Js[ns * n + k] = (m->mw[k] / rho) * (JTa[k] + tka / T);
  }
  /* temperature row */
  double HS = 0.0, HSa = 0.0;
  for (int k = 0; k < ns; ++k) { HS += hRT[k] * S[k]; HSa += fabs(hRT[k]) * Sa[k]; }
  for (int mm = 0; mm < ns; ++mm) {
    double HJ = 0.0, HJa = 0.0;
    for (int k = 0; k < ns; ++k) { HJ += hRT[k] * Jc[mm * ns + k]; HJa += fabs(hRT[k]) * Jca[mm * ns + k]; }
    double dQ = (rho / m->mw[mm]) * HJ - (wbar / m->mw[mm]) * HS;
    double dQa = (rho / m->mw[mm]) * HJa + (wbar / m->mw[mm]) * HSa;
    double dD = (rho / m->mw[mm]) * cpR[mm] - (wbar / m->mw[mm]) * D;
    double dDa = (rho / m->mw[mm]) * fabs(cpR[mm]) + (wbar / m->mw[mm]) * fabs(D);
    J[mm * n + ns] = -(T / D) * (dQ - (Q / D) * dD);
    if (Js) Js[mm * n + ns] = (T / fabs(D)) * (dQa + (Qa / fabs(D)) * dDa);
  }
  {
    double dQT = 0.0, dQTa = 0.0, dDT = 0.0, dDTa = 0.0;
    for (int k = 0; k < ns; ++k) {
      dQT += (cpR[k] - hRT[k]) / T * wm[k] + hRT[k] * (JT[k] - S[k] / T);
      dQTa += fabs((cpR[k] - hRT[k]) / T) * wabs[k] + fabs(hRT[k]) * (JTa[k] + Sa[k] / T);
      dDT += c[k] * (dcpR[k] - cpR[k] / T);
      dDTa += fabs(c[k]) * (fabs(dcpR[k]) + fabs(cpR[k]) / T);
    }
    J[ns * n + ns] = -Q / D - (T / D) * (dQT - (Q / D) * dDT);
    if (Js) Js[ns * n + ns] = Qa / fabs(D) + (T / fabs(D)) * (dQTa + (Qa / fabs(D)) * dDTa);
  }
  free(Jc);
}

/* Constant volume: the system rhs_native integrates (Lib_Chemistry_rhs.f90:
 * 15-52: rho fixed, energy equation :43-50) with the analytic mechanism.
 * c_k = rho Y_k / W_k, dY_k/dt = W_k wdot_k / rho and, per mole,
 * dT/dt = -sum_k (h_k - R T) wdot_k / (sum_k c_k (cp_k - R)). */
void orc_rhs_constv_cell(const flint_mech_desc* m, double T, double rho, const double* Y, double* f) {
  int ns = m->ns;
  double c[MAXNS], cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS], wm[MAXNS], wabs[MAXNS];
  for (int k = 0; k < ns; ++k) c[k] = rho * Y[k] / m->mw[k];
  orc_species_thermo(m, T, cpR, hRT, sR, NULL);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  kinetics(m, T, c, hRT, gRT, wm, wabs, NULL, NULL, NULL, NULL);
  double Q = 0.0, D = 0.0;
  for (int k = 0; k < ns; ++k) {
    f[k] = m->mw[k] * wm[k] / rho;
    Q += (hRT[k] - 1.0) * wm[k];
    D += c[k] * (cpR[k] - 1.0);
  }
  f[ns] = -T * Q / D;
}

/* d(dY/dt, dT/dt)/d(Y, T) at fixed rho (column-major per cell like
 * orc_jac_cell; Js the same chain rule on term magnitudes). */
void orc_jac_constv_cell(const flint_mech_desc* m, double T, double rho, const double* Y,
                         double* f, double* J, double* Js) {
  int ns = m->ns, n = ns + 1;
  double c[MAXNS], cpR[MAXNS], hRT[MAXNS], sR[MAXNS], gRT[MAXNS], dcpR[MAXNS];
  double wm[MAXNS], wabs[MAXNS], JT[MAXNS], JTa[MAXNS];
  double* Jc = (double*)malloc(sizeof(double) * ns * ns * 2);
  double* Jca = Jc + ns * ns;
  for (int k = 0; k < ns; ++k) c[k] = rho * Y[k] / m->mw[k];
  orc_species_thermo(m, T, cpR, hRT, sR, dcpR);
  for (int k = 0; k < ns; ++k) gRT[k] = hRT[k] - sR[k];
  kinetics(m, T, c, hRT, gRT, wm, wabs, Jc, Jca, JT, JTa);
  double Q = 0.0, Qa = 0.0, D = 0.0;
  for (int k = 0; k < ns; ++k) {
    Q += (hRT[k] - 1.0) * wm[k];
    Qa += fabs(hRT[k] - 1.0) * wabs[k];
    D += c[k] * (cpR[k] - 1.0);
  }
  for (int k = 0; k < ns; ++k) f[k] = m->mw[k] * wm[k] / rho;
  f[ns] = -T * Q / D;
  /* species rows: dc_j/dY_mm = rho/W_mm delta_j,mm, dc/dT = 0 */
  for (int k = 0; k < ns; ++k) {
    for (int mm = 0; mm < ns; ++mm) {
      double ratio = m->mw[k] / m->mw[mm];
      J[mm * n + k] = ratio * Jc[mm * ns + k];
      if (Js) Js[mm * n + k] = ratio * Jca[mm * ns + k];
    }
    J[ns * n + k] = (m->mw[k] / rho) * JT[k];
    if (Js) Js[ns * n + k] = (m->mw[k] / rho) * JTa[k];
  }
  /* temperature row */
  for (int mm = 0; mm < ns; ++mm) {
    double HJ = 0.0, HJa = 0.0;
    for (int k = 0; k < ns; ++k) {
      HJ += (hRT[k] - 1.0) * Jc[mm * ns + k];
      HJa += fabs(hRT[k] - 1.0) * Jca[mm * ns + k];
    }
    double rw = rho / m->mw[mm];
    double dQ = rw * HJ, dQa = rw * HJa;
    double dD = rw * (cpR[mm] - 1.0), dDa = rw * fabs(cpR[mm] - 1.0);
    J[mm * n + ns] = -(T / D) * (dQ - (Q / D) * dD);
    if (Js) Js[mm * n + ns] = (T / fabs(D)) * (dQa + (Qa / fabs(D)) * dDa);
  }
  {
    double dQT = 0.0, dQTa = 0.0, dDT = 0.0, dDTa = 0.0;
    for (int k = 0; k < ns; ++k) {
      dQT += (cpR[k] - hRT[k]) / T * wm[k] + (hRT[k] - 1.0) * JT[k];
      dQTa += fabs((cpR[k] - hRT[k]) / T) * wabs[k] + fabs(hRT[k] - 1.0) * JTa[k];
      dDT += c[k] * dcpR[k];
      dDTa += fabs(c[k]) * fabs(dcpR[k]);
    }
    J[ns * n + ns] = -Q / D - (T / D) * (dQT - (Q / D) * dDT);
    if (Js) Js[ns * n + ns] = Qa / fabs(D) + (T / fabs(D)) * (dQTa + (Qa / fabs(D)) * dDTa);
  }
  free(Jc);
}

void orc_jac_constv_batch(const flint_mech_desc* m, int64_t n, const double* T, const double* rho,
                          const double* Y, double* f, double* jac, double* jscale, int nthreads) {
  int ns = m->ns, nv = ns + 1, nn = nv * nv;
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double fl[MAXNS + 1];
    orc_jac_constv_cell(m, T[i], rho[i], Y + i * ns, fl, jac + i * nn, jscale ? jscale + i * nn : NULL);
    if (f) for (int k = 0; k < nv; ++k) f[i * nv + k] = fl[k];
  }
}

/* ------------------------------------------------------------------ batches */
static void gather_Y(int64_t i, int64_t n, int ns, int layout, const double* Y, double* y) {
  for (int k = 0; k < ns; ++k) y[k] = (layout == FLINT_SPECIES_MAJOR) ? Y[(int64_t)k * n + i] : Y[i * ns + k];
}

void orc_wdot_batch(const flint_mech_desc* m, int64_t n, int layout, const double* T,
                    const double* p, const double* Y, double* wdot, double* wscale,
                    double* cp, double* h, int nthreads) {
  int ns = m->ns;
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double y[MAXNS], w[MAXNS], ws[MAXNS], cpv, hv;
    gather_Y(i, n, ns, layout, Y, y);
    orc_wdot_cell(m, T[i], p[i], y, w, ws, &cpv, &hv);
    for (int k = 0; k < ns; ++k) {
      int64_t idx = (layout == FLINT_SPECIES_MAJOR) ? (int64_t)k * n + i : i * ns + k;
      if (wdot) wdot[idx] = w[k];
      if (wscale) wscale[idx] = ws[k];
    }
    if (cp) cp[i] = cpv;
    if (h) h[i] = hv;
  }
}

void orc_wdot_jac_batch(const flint_mech_desc* m, int64_t n, int layout, const double* T,
                        const double* p, const double* Y, double* wdot, double* jac,
                        double* jscale, int nthreads) {
  int ns = m->ns, nn = (ns + 1) * (ns + 1);
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double y[MAXNS], f[MAXNS + 1];
    gather_Y(i, n, ns, layout, Y, y);
    if (wdot) {
      double w[MAXNS];
      orc_wdot_cell(m, T[i], p[i], y, w, NULL, NULL, NULL);
      for (int k = 0; k < ns; ++k) {
        int64_t idx = (layout == FLINT_SPECIES_MAJOR) ? (int64_t)k * n + i : i * ns + k;
        wdot[idx] = w[k];
      }
    }
    orc_jac_cell(m, T[i], p[i], y, f, jac + i * nn, jscale ? jscale + i * nn : NULL);
  }
}

/* ------------------------------------------------------------------ reactor */
/* Nordsieck BDF coefficients: l^(q)_j = coefficient of x^j in prod_{i=1..q}(1 + x/i). */
static void bdf_l(int q, double* l) {
  for (int j = 0; j <= 5; ++j) l[j] = 0.0;
  l[0] = 1.0;
  for (int i = 1; i <= q; ++i)
    for (int j = i; j >= 1; --j) l[j] += l[j - 1] / (double)i;
}

static double wrms(int n, const double* v, const double* w) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) { double t = v[i] * w[i]; s += t * t; }
  return sqrt(s / n);
}

/* Weighted max norm: the Newton convergence test, so that no single
 * component (a trace radical at atol) can stay unconverged behind the RMS. */
static double wmax(int n, const double* v, const double* w) {
  double m = 0.0;
  for (int i = 0; i < n; ++i) { double t = fabs(v[i] * w[i]); if (t > m) m = t; }
  return m;
}

/* LU with partial pivoting (first maximal |a| on ties), in place, column-major. */
static int lu_factor(int n, double* a, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k; double amax = fabs(a[k * n + k]);
    for (int i = k + 1; i < n; ++i) { double v = fabs(a[k * n + i]); if (v > amax) { amax = v; p = i; } }
    piv[k] = p;
    if (amax == 0.0) return 1;
    if (p != k) for (int j = 0; j < n; ++j) { double t = a[j * n + k]; a[j * n + k] = a[j * n + p]; a[j * n + p] = t; }
    double inv = 1.0 / a[k * n + k];
    a[k * n + k] = inv;   /* U's diagonal kept as its reciprocal: solves multiply */
    for (int i = k + 1; i < n; ++i) a[k * n + i] *= inv;
    for (int j = k + 1; j < n; ++j) {
      double akj = a[j * n + k];
      for (int i = k + 1; i < n; ++i) a[j * n + i] -= a[k * n + i] * akj;
    }
  }
  return 0;
}

static void lu_solve(int n, const double* a, const int* piv, double* b) {
  for (int k = 0; k < n; ++k) { int p = piv[k]; if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; } }
  for (int k = 0; k < n; ++k) for (int i = k + 1; i < n; ++i) b[i] -= a[k * n + i] * b[k];
  for (int k = n - 1; k >= 0; --k) {
    b[k] *= a[k * n + k];
    for (int i = 0; i < k; ++i) b[i] -= a[k * n + i] * b[k];
  }
}

/* p: pressure (constant pressure) or density (constv: constant volume) */
typedef struct { const flint_mech_desc* m; double p; int constv; } rhs_ctx;

static void rhs_y(const rhs_ctx* cx, const double* y, double* f) {
  int ns = cx->m->ns;
  if (cx->constv) orc_rhs_constv_cell(cx->m, y[ns], cx->p, y, f);
  else orc_rhs_constp_cell(cx->m, y[ns], cx->p, y, f);
}

static void jac_y(const rhs_ctx* cx, const double* y, double* J) {
  int ns = cx->m->ns;
  double f[MAXNS + 1];
  if (cx->constv) orc_jac_constv_cell(cx->m, y[ns], cx->p, y, f, J, NULL);
  else orc_jac_cell(cx->m, y[ns], cx->p, y, f, J, NULL);
}

/* One cell of the reactor.  Returns the FLINT_CELL_* status.  The step-size
 * factors eta = (c*dsm)^(-1/(q+1)) are heuristics evaluated in FP32, as the GPU
 * does; the solution itself is FP64 throughout. */
static int bdf_cell(const rhs_ctx* cx, int n, double* y, double tout, const flint_reactor_opts* o,
                    int* nsteps_out) {
  double z[6][MAXNS + 1], zs[6][MAXNS + 1];
  double e[MAXNS + 1], eprev[MAXNS + 1], ewt[MAXNS + 1], ypred[MAXNS + 1], f[MAXNS + 1], b[MAXNS + 1];
  double* J = (double*)malloc(sizeof(double) * n * n * 2);
  double* Mlu = J + n * n;
  int piv[MAXNS + 1];
  double L[6][6];
  for (int q = 1; q <= 5; ++q) bdf_l(q, L[q]);
  int qmax = o->max_order < 1 ? 1 : (o->max_order > 5 ? 5 : o->max_order);
  double rtol = o->rtol, atol = o->atol;
  int status = FLINT_CELL_OK;
  int nst = 0;

  for (int i = 0; i < n; ++i) z[0][i] = y[i];
  rhs_y(cx, y, f);
  for (int i = 0; i < n; ++i) ewt[i] = 1.0 / (rtol * fabs(y[i]) + atol);
  double fn = wrms(n, f, ewt);
  double h = (fn * tout > 1.0) ? 1.0 / fn : tout;
  for (int i = 0; i < n; ++i) z[1][i] = h * f[i];
  int q = 1;
  double t = 0.0;
  int ialth = 2;            /* steps until the next step-size / order decision */
  int have_J = 0, jfresh = 0;
  double gammaJ = 0.0;
  int nstJ = 0, nstP = 0;
  double crate = 1.0;
  double etamax = 1.0e4;
  int have_eprev = 0;
  int last = 0;

  while (t < tout) {
    if (nst >= o->max_steps) { status = FLINT_CELL_MAX_STEPS; break; }
    /* land exactly on tout */
    last = 0;
    if (t + h >= tout) {
      double eta = (tout - t) / h;
      double r = 1.0;
      for (int j = 1; j <= q; ++j) { r *= eta; for (int i = 0; i < n; ++i) z[j][i] *= r; }
      h = tout - t;
      ialth = q + 1; have_eprev = 0;
      last = 1;
    }
    for (int i = 0; i < n; ++i) ewt[i] = 1.0 / (rtol * fabs(z[0][i]) + atol);
    int ncf = 0, nef = 0, need_J = 0;
    double dsm = 0.0;
    /* the first Newton iterate of a step is judged with a rate of at least 0.3:
     * a small rate carried over from the last step would accept it unchecked */
    if (crate < 0.3) crate = 0.3;
    int accepted = 0;
    while (!accepted) {
      if (h < 1e-300 || t + h == t) { status = FLINT_CELL_ERRTEST_FAIL; break; }
      /* save and predict */
      for (int j = 0; j <= q; ++j) for (int i = 0; i < n; ++i) zs[j][i] = z[j][i];
      for (int k = 0; k < q; ++k)
        for (int j = q - 1; j >= k; --j)
          for (int i = 0; i < n; ++i) z[j][i] += z[j + 1][i];
      double l1 = L[q][1];
      double gamma = h / l1;
      for (int i = 0; i < n; ++i) ypred[i] = z[0][i];
      /* Newton matrix refresh (gamma moved > 30 % or 20 steps) and Jacobian
       * re-evaluation (50 steps or a failure with a stale one): CVODE's policy. */
      if (!have_J || need_J || fabs(gamma / gammaJ - 1.0) > 0.3 || nst >= nstP + 20) {
        if (!have_J || need_J || nst >= nstJ + 50) {
          jac_y(cx, ypred, J);
          have_J = 1; jfresh = 1; nstJ = nst; need_J = 0;
        }
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) Mlu[j * n + i] = (i == j ? 1.0 : 0.0) - gamma * J[j * n + i];
        lu_factor(n, Mlu, piv);
        gammaJ = gamma; nstP = nst; crate = 1.0;
      }
      double gamrat = gamma / gammaJ;
      /* Newton iteration on e = y - ypred */
      for (int i = 0; i < n; ++i) { e[i] = 0.0; y[i] = ypred[i]; }
      int conv = 0;
      double delp = 0.0;
      double Eq = 1.0 / ((double)(q + 1) * l1 + 1.0);
      double il1 = 1.0 / l1;
      for (int mi = 0; mi < 3; ++mi) {
        rhs_y(cx, y, f);
        for (int i = 0; i < n; ++i) b[i] = gamma * f[i] - z[1][i] * il1 - e[i];
        lu_solve(n, Mlu, piv, b);
        if (gamrat != 1.0) { double s = 2.0 / (1.0 + gamrat); for (int i = 0; i < n; ++i) b[i] *= s; }
        double del = wmax(n, b, ewt);
        for (int i = 0; i < n; ++i) { e[i] += b[i]; y[i] = ypred[i] + e[i]; }
        if (mi > 0) { double r = del / delp; crate = (0.3 * crate > r) ? 0.3 * crate : r; }
        double dcon = del * (crate < 1.0 ? crate : 1.0) * Eq * 10.0;   /* test constant 0.1 */
        if (dcon <= 1.0) { conv = 1; break; }
        if (mi > 0 && !(del <= 2.0 * delp)) break;
        delp = del;
      }
      if (!conv) {
        for (int j = 0; j <= q; ++j) for (int i = 0; i < n; ++i) z[j][i] = zs[j][i];
        ++ncf;
        if (ncf >= 10) { status = FLINT_CELL_NEWTON_FAIL; break; }
        if (!jfresh) { need_J = 1; continue; }
        double eta = 0.25, r = 1.0;
        for (int j = 1; j <= q; ++j) { r *= eta; for (int i = 0; i < n; ++i) z[j][i] *= r; }
        h *= eta; ialth = q + 1; have_eprev = 0; need_J = 1; last = 0;
        continue;
      }
      dsm = Eq * wrms(n, e, ewt);
      if (!(dsm <= 1.0)) {
        for (int j = 0; j <= q; ++j) for (int i = 0; i < n; ++i) z[j][i] = zs[j][i];
        ++nef;
        if (nef >= 7) { status = FLINT_CELL_ERRTEST_FAIL; break; }
        double eta;
        if (nef >= 3) {
          eta = 0.1;
          if (q > 1) q = 1;
        } else {
          eta = 1.0 / ((double)powf((float)(1.2 * dsm), 1.0f / (float)(q + 1)) + 1e-6);
          if (eta > 0.9) eta = 0.9;
          if (eta < 0.1) eta = 0.1;
        }
        double r = 1.0;
        for (int j = 1; j <= q; ++j) { r *= eta; for (int i = 0; i < n; ++i) z[j][i] *= r; }
        h *= eta; ialth = q + 1; have_eprev = 0; last = 0;
        if (!jfresh) need_J = 1;   /* retry with a Jacobian of this state */
        continue;
      }
      accepted = 1;
    }
    if (status != FLINT_CELL_OK) break;
    /* accept: correct the Nordsieck array */
    t += h;
    ++nst;
    jfresh = 0;
    for (int j = 0; j <= q; ++j) for (int i = 0; i < n; ++i) z[j][i] += L[q][j] * e[i];
    if (last || t >= tout) { t = tout; break; }
    --ialth;
    double eta = 1.0;
    if (ialth <= 0) {
      double l1 = L[q][1];
      double etaq = 1.0 / ((double)powf((float)(1.2 * dsm), 1.0f / (float)(q + 1)) + 1.2e-6);
      double etadn = 0.0, etaup = 0.0;
      if (q > 1) {
        double fact = 1.0;
        for (int i = 2; i <= q; ++i) fact *= i;
        double ddn = wrms(n, z[q], ewt) * fact / ((double)q * L[q - 1][1]);
        etadn = 1.0 / ((double)powf((float)(1.3 * ddn), 1.0f / (float)q) + 1.3e-6);
      }
      if (q < qmax && have_eprev) {
        double d[MAXNS + 1];
        for (int i = 0; i < n; ++i) d[i] = e[i] - eprev[i];
        double Kq = 1.0 + 1.0 / ((double)(q + 1) * l1);
        double dup = wrms(n, d, ewt) / (Kq * (double)(q + 2) * L[q + 1][1]);
        etaup = 1.0 / ((double)powf((float)(1.4 * dup), 1.0f / (float)(q + 2)) + 1.4e-6);
      }
      int newq = q;
      eta = etaq;
      if (etaup > eta && etaup >= etadn) { eta = etaup; newq = q + 1; }
      else if (etadn > eta) { eta = etadn; newq = q - 1; }
      if (newq == q + 1) {
        double fct = L[q][q] / (double)(q + 1);
        for (int i = 0; i < n; ++i) z[q + 1][i] = e[i] * fct;
      }
      if (eta < 1.1 && newq == q) {
        eta = 1.0;
        ialth = 3;
      } else {
        q = newq;
        if (eta > etamax) eta = etamax;
        ialth = q + 1;
      }
      have_eprev = 0;
      etamax = 10.0;
    } else if (ialth == 1 && q < qmax) {
      for (int i = 0; i < n; ++i) eprev[i] = e[i];
      have_eprev = 1;
    }
    if (eta != 1.0) {
      double r = 1.0;
      for (int j = 1; j <= q; ++j) { r *= eta; for (int i = 0; i < n; ++i) z[j][i] *= r; }
      h *= eta;
    }
  }
  for (int i = 0; i < n; ++i) y[i] = z[0][i];
  if (nsteps_out) *nsteps_out = nst;
  free(J);
  return status;
}

/* A cell whose integration fails (error test or Newton) is integrated again
 * from its initial state, first at order <= 2 with atol / 100 (BDF1-2 are
 * A-stable; orders 3-5 are not, and a mechanism's oscillatory modes can defeat
 * them), then at order 1.  nsteps counts the steps of every attempt. */
static int reactor_cell(const rhs_ctx* cx, int n, double* y, double tout, const flint_reactor_opts* o,
                        int* nsteps_out) {
  double y0[MAXNS + 1];
  for (int i = 0; i < n; ++i) y0[i] = y[i];
  int total = 0, st = FLINT_CELL_OK;
  for (int att = 0; att < 3; ++att) {
    flint_reactor_opts oa = *o;
    if (att == 1) { if (oa.max_order > 2) oa.max_order = 2; oa.atol *= 1e-2; }
    if (att == 2) oa.max_order = 1;
    if (att > 0) for (int i = 0; i < n; ++i) y[i] = y0[i];
    int nst = 0;
    st = bdf_cell(cx, n, y, tout, &oa, &nst);
    total += nst;
    if (st != FLINT_CELL_ERRTEST_FAIL && st != FLINT_CELL_NEWTON_FAIL) break;
  }
  *nsteps_out = total;
  return st;
}

void orc_reactor_advance(const flint_mech_desc* m, int64_t n, double* T, const double* p,
                         double* Y, const double* dt, const flint_reactor_opts* o,
                         int* status, int* nsteps, int nthreads) {
  int ns = m->ns;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    double y[MAXNS + 1];
    int st, nst = 0;
    for (int k = 0; k < ns; ++k) y[k] = Y[i * ns + k];
    y[ns] = T[i];
    int bad = !(isfinite(T[i]) && isfinite(p[i]) && p[i] > 0.0 && isfinite(dt[i]) && dt[i] >= 0.0);
    for (int k = 0; k < ns; ++k) bad |= !isfinite(y[k]);
    if (bad) st = FLINT_CELL_NAN_INPUT;
    else if (T[i] < o->tmin || T[i] > o->tmax) st = FLINT_CELL_T_OUT_OF_RANGE;
    else if (dt[i] == 0.0) st = FLINT_CELL_OK;
    else {
      double pr = p[i];
      if (o->constant_volume) {   /* density fixed at its initial value */
        double sumYW = 0.0;
        for (int k = 0; k < ns; ++k) sumYW += y[k] / m->mw[k];
        pr = p[i] / (m->r_eos * T[i] * sumYW);
      }
      rhs_ctx cx = {m, pr, o->constant_volume};
      st = reactor_cell(&cx, ns + 1, y, dt[i], o, &nst);
      for (int k = 0; k < ns; ++k) Y[i * ns + k] = y[k];
      T[i] = y[ns];
    }
    if (status) status[i] = st;
    if (nsteps) nsteps[i] = nst;
  }
}

/* ------------------------------------------------------- TABLE mode (reference) */
/* comp_ch_tabT: a + (b-a)*Tdiff on rows T_i, T_i+1 (Lib_Chemistry_data.f90:36-48). */
static double lerp_tab(const double* tab, int row0, int nrows, int col, int Ti, double Tdiff) {
  int row = Ti - row0;   /* edge rows outside the table (the reference reads past it) */
  row = row < 0 ? 0 : (row > nrows - 2 ? nrows - 2 : row);
  double a = tab[(int64_t)col * nrows + row];
  double b = tab[(int64_t)col * nrows + row + 1];
  return a + (b - a) * Tdiff;
}

/* Fortran coi**nint(x) with integer exponent: repeated multiplication. */
static double ipow_f(double x, int n) {
  if (n == 0) return 1.0;
  int neg = n < 0; if (neg) n = -n;
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return neg ? 1.0 / r : r;
}

/* f_F (Lib_Chemistry_falloff.f90:61-80). */
static double troe_F(double Pr, double Fcent) {
  double logFcent = log10(Fcent);
  double logPr = log10(Pr);
  double c = -0.4 - 0.67 * logFcent;
  double nn = 0.75 - 1.27 * logFcent;
  double f1 = (logPr + c) / (nn - 0.14 * (logPr + c));
  return pow(10.0, logFcent / (1.0 + f1 * f1));
}

void orc_general(const orc_table_mech* m, const double* roi, double temp, double* omegadot) {
  int ns = m->ns, nrows = m->ti2 - m->ti1 + 1;
  double coi[MAXNS];
  for (int s = 0; s < ns; ++s) coi[s] = roi[s] / m->wm[s];
  int Ti = (int)temp;
  double Tdiff = temp - Ti;
  for (int s = 0; s < ns; ++s) omegadot[s] = 0.0;
  for (int kind = 0; kind < 3; ++kind) {
    int nr = kind == 0 ? m->nr_arrh : (kind == 1 ? m->nr_troe : m->nr_lind);
    const double* ni1 = kind == 0 ? m->ni1_arrh : (kind == 1 ? m->ni1_troe : m->ni1_lind);
    const double* ni2 = kind == 0 ? m->ni2_arrh : (kind == 1 ? m->ni2_troe : m->ni2_lind);
    const double* eps = kind == 0 ? m->eps_arrh : (kind == 1 ? m->eps_troe : m->eps_lind);
    for (int ir = 0; ir < nr; ++ir) {
      const double* n1 = ni1 + (int64_t)ir * (ns + 1);
      const double* n2 = ni2 + (int64_t)ir * (ns + 1);
      const double* ep = eps + (int64_t)ir * (ns + 1);
      double coM;
      if (n1[ns] > 0.0) {
        coM = 0.0;
        for (int s = 0; s < ns; ++s) coM = coM + coi[s] * ep[s];
      } else {
        coM = 1.0;
      }
      double prod_fwd = 1.0, prod_rev = 1.0, rate_fwd, rate_rev;
      if (kind == 0) {
        for (int s = 0; s < ns; ++s) {
          if (n1[s] != 0.0) prod_fwd = prod_fwd * ipow_f(coi[s], (int)lround(n1[s]));
          if (n2[s] != 0.0) prod_rev = prod_rev * ipow_f(coi[s], (int)lround(n2[s]));
        }
        rate_fwd = lerp_tab(m->kf_tab, m->ti1, nrows, ir, Ti, Tdiff) * prod_fwd * coM;
        rate_rev = lerp_tab(m->kb_tab, m->ti1, nrows, ir, Ti, Tdiff) * prod_rev * coM;
      } else {
        /* real powers: coi**ni (Lib_Chemistry_wdot.f90:166-167, :200-201) */
        for (int s = 0; s < ns; ++s) {
          if (n1[s] != 0.0) prod_fwd = prod_fwd * pow(coi[s], n1[s]);
          if (n2[s] != 0.0) prod_rev = prod_rev * pow(coi[s], n2[s]);
        }
        double kinf, k0, kc, k1;
        if (kind == 1) {
          kinf = lerp_tab(m->kinf_troe, m->ti1, nrows, ir, Ti, Tdiff);
          k0 = lerp_tab(m->k0_troe, m->ti1, nrows, ir, Ti, Tdiff);
          kc = lerp_tab(m->kc_troe, m->ti1, nrows, ir, Ti, Tdiff);
          double Fcent = lerp_tab(m->fcent_troe, m->ti1, nrows, ir, Ti, Tdiff);
          double Pr = k0 * coM / kinf;
          k1 = kinf * (Pr / (1.0 + Pr)) * troe_F(Pr, Fcent);
        } else {
          kinf = lerp_tab(m->kinf_lind, m->ti1, nrows, ir, Ti, Tdiff);
          k0 = lerp_tab(m->k0_lind, m->ti1, nrows, ir, Ti, Tdiff);
          kc = lerp_tab(m->kc_lind, m->ti1, nrows, ir, Ti, Tdiff);
          double Pr = k0 * coM / kinf;
          k1 = kinf * (Pr / (1.0 + Pr));
        }
        rate_fwd = k1 * prod_fwd;
        rate_rev = (k1 / kc) * prod_rev;
      }
      double net_rate = rate_fwd - rate_rev;
      for (int s = 0; s < ns; ++s) {
        double deltani = n2[s] - n1[s];
        omegadot[s] = omegadot[s] + m->wm[s] * deltani * net_rate;
      }
    }
  }
}

void orc_rhs_native(const orc_table_mech* m, int nz, const double* Z, double* F) {
  int ns = m->ns, nrows = m->tmax - m->tmin + 1;
  double roi[MAXNS], droic[MAXNS];
  for (int s = 0; s < ns; ++s) roi[s] = Z[s];
  double T = Z[nz - 1];
  if (T < m->tmin || T > m->tmax || isnan(T)) {
    for (int i = 0; i < nz; ++i) F[i] = -1.0;
    return;
  }
  for (int s = 0; s < ns; ++s) roi[s] = roi[s] > 0.0 ? roi[s] : 0.0;
  orc_general(m, roi, T, droic);
  int Ti = (int)T;
  double Tdiff = T - Ti;
  double eiroi = 0.0, rho_cv = 0.0;
  for (int s = 0; s < ns; ++s) {
    double hs = lerp_tab(m->h_tab, m->tmin, nrows, s, Ti, Tdiff);
    double cps = lerp_tab(m->cp_tab, m->tmin, nrows, s, Ti, Tdiff);
    double ri = m->runiv / m->wm[s];   /* Ri_tab = Runiv/wm_tab, Load_ThermoTransport.f90:54 */
    eiroi = eiroi + (hs - ri * T) * droic[s];
    rho_cv = rho_cv + roi[s] * (cps - ri);
  }
  for (int s = 0; s < ns; ++s) F[s] = droic[s];
  F[nz - 1] = -eiroi / rho_cv;
}

void orc_general_batch(const orc_table_mech* m, int64_t n, const double* roi, const double* T,
                       double* omegadot, int nthreads) {
  int ns = m->ns;
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) orc_general(m, roi + i * ns, T[i], omegadot + i * ns);
}

void orc_rhs_native_batch(const orc_table_mech* m, int64_t n, const double* Z, double* F,
                          int nthreads) {
  int nz = m->ns + 1;
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) orc_rhs_native(m, nz, Z + i * nz, F + i * nz);
}

/* ------------------------------------------------------------- cons2prim */
/* norm2 as gfortran evaluates it: a scaled sum of squares (overflow-safe). */
static double norm2_f(int n, const double* x) {
  double scale = 1.0, ssq = 0.0;
  for (int i = 0; i < n; ++i) {
    if (x[i] != 0.0) {
      double a = fabs(x[i]);
      if (scale < a) {
        double v = scale / a;
        ssq = 1.0 + ssq * v * v;
        scale = a;
      } else {
        double v = a / scale;
        ssq = ssq + v * v;
      }
    }
  }
  return scale * sqrt(ssq);
}

static double sum_f(int n, const double* x) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s = s + x[i];
  return s;
}

/* f_Rtot (Lib_ThermoTransport.f90:217-230): sum_s Ri_s rhoi_s / rho. */
static double rtot_f(const orc_table_mech* m, const double* r) {
  double rho = sum_f(m->ns, r), res = 0.0;
  for (int s = 0; s < m->ns; ++s) res = res + (m->runiv / m->wm[s]) * r[s] / rho;
  return res;
}

/* f_cp (Lib_ThermoTransport.f90:251-271): sum_s rhoi_s / rho * cp_s(T). */
static double cp_f(const orc_table_mech* m, const double* r, double T, double rho) {
  int nrows = m->tmax - m->tmin + 1, Ti = (int)T;
  double Tdiff = T - Ti, res = 0.0;
  for (int s = 0; s < m->ns; ++s) res = res + r[s] / rho * lerp_tab(m->cp_tab, m->tmin, nrows, s, Ti, Tdiff);
  return res;
}

/* H (Lib_ThermoTransport.f90:40-54) with f_tab's T = p / (Rtot rho) (:500-512). */
static double h_f(const orc_table_mech* m, double p, const double* r) {
  int nrows = m->tmax - m->tmin + 1;
  double rho = sum_f(m->ns, r), Rgas = rtot_f(m, r), res = 0.0;
  double T = p / (Rgas * rho);
  int Ti = (int)T;
  double Tdiff = T - Ti;
  for (int s = 0; s < m->ns; ++s) res = res + lerp_tab(m->h_tab, m->tmin, nrows, s, Ti, Tdiff) * r[s] / rho;
  return res;
}

/* cons2prim (Lib_ThermoTransport.f90:129-165): cons = (rho_s, rho u_d, rho E0),
 * prim = (rho_s, u_d, p); T is the Newton start and *Tout the last iterate. */
void orc_cons2prim(const orc_table_mech* m, int np, const double* cons, double T, double* prim,
                   double* Tout, int* iters) {
  int ns = m->ns, nui = ns, nuf = np - 2;   /* 0-based: velocity slots nui..nuf */
  double rhoi[MAXNS];
  for (int s = 0; s < ns; ++s) rhoi[s] = cons[s];
  double Rgas = rtot_f(m, rhoi);
  double rho = sum_f(ns, rhoi);
  for (int s = 0; s < ns; ++s) prim[s] = rhoi[s];
  for (int d = nui; d <= nuf; ++d) prim[d] = cons[d] / rho;
  double vel = norm2_f(nuf - nui + 1, prim + nui);
  double energy = cons[np - 1] / rho - 0.5 * vel * vel;
  double diff_en = 1.0e3, T_iter = T;
  int it = 1;
  while (fabs(diff_en / energy) >= 1e-6 && it <= 20) {
    double p_iter = rho * Rgas * T_iter;
    double cv_iter = cp_f(m, rhoi, T_iter, rho) - Rgas;
    double energy_iter = h_f(m, p_iter, rhoi) - p_iter / sum_f(ns, rhoi);
    diff_en = fabs(energy_iter - energy);
    T_iter = T_iter + (energy - energy_iter) / cv_iter;
    it = it + 1;
  }
  prim[np - 1] = rho * Rgas * T_iter;
  if (Tout) *Tout = T_iter;
  if (iters) *iters = it - 1;
}

void orc_cons2prim_batch(const orc_table_mech* m, int64_t n, int np, const double* cons,
                         const double* T, double* prim, double* Tout, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    orc_cons2prim(m, np, cons + i * np, T[i], prim + i * np, Tout ? Tout + i : NULL, NULL);
}

/* ------------------------------------------------------------- transport */
/* f_molecularWeight (Lib_ThermoTransport.f90:200-214): 1 / sum_s rhoi_s / rho / W_s. */
static double wmol_f(const orc_table_mech* m, const double* r) {
  double rho = sum_f(m->ns, r), res = 0.0;
  for (int s = 0; s < m->ns; ++s) res = res + r[s] / rho / m->wm[s];
  return 1.0 / res;
}

/* co_k_mi_lam_Wilke(rhoi, rho, T, milam, klam), Lib_ThermoTransport.f90:407-462,
 * with its co_fiij (:350-362): Wilke's mixing rule on the tabulated species
 * viscosities and conductivities. */
void orc_transport(const orc_table_mech* m, const double* rhoi, double T, double* mu, double* lam) {
  int ns = m->ns, nrows = m->tmax - m->tmin + 1, Ti = (int)T;
  double Tdiff = T - Ti;
  double rho = sum_f(ns, rhoi);
  double Wmtot = wmol_f(m, rhoi);
  double Xi[MAXNS], mi[MAXNS], ki[MAXNS], den[MAXNS];
  for (int s = 0; s < ns; ++s) {
    Xi[s] = rhoi[s] * Wmtot / (rho * m->wm[s]);
    mi[s] = lerp_tab(m->mi_tab, m->tmin, nrows, s, Ti, Tdiff);
    ki[s] = lerp_tab(m->k_tab, m->tmin, nrows, s, Ti, Tdiff);
  }
  for (int i = 0; i < ns; ++i) {
    den[i] = 0.0;
    for (int j = 0; j < ns; ++j) {
      double MiMj = m->wm[i] / m->wm[j];
      double a = 1.0 + sqrt(mi[i] / (mi[j] + 1e-20)) / pow(MiMj, 0.25);
      double fi = a * a / sqrt(8.0 * (1.0 + MiMj));
      den[i] = den[i] + Xi[j] * fi;
    }
  }
  double mil = 0.0, kl = 0.0;
  for (int s = 0; s < ns; ++s) {
    double inv = 1.0 / den[s];
    mil = mil + Xi[s] * mi[s] * inv;
    kl = kl + Xi[s] * ki[s] * inv;
  }
  *mu = mil;
  *lam = kl;
}

void orc_transport_batch(const orc_table_mech* m, int64_t n, const double* rhoi, const double* T, double* mu,
                         double* lam, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) orc_transport(m, rhoi + i * m->ns, T[i], mu + i, lam + i);
}
