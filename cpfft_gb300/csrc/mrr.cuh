// mrr.cuh -- dislocation-density hardening for the stress kernel: twelve dislocation
// densities, one per slip system of a 12-system crystal, as the slip resistance
// variables.  Ma-Roters-Raabe (h_type 7, stress_mrr.cu) and ORNL (h_type 4,
// stress_ornl.cu: the same hardening law with the temperature-dependent shear modulus
// mu(T) = mu_0 - D_0 / (exp(T_0 / T) - 1),
// and its own slip law, mm10_slipinc_ornl .. mm10_dgdh_ornl, src/mm10_b.f:3457-4347).
// Included by stress.cu when it is compiled with CPFFT_LAW 7 or 4.
//
// The slip law, hardening law and their derivatives follow mm10_slipinc_mrr ..
// mm10_dgdd_mrr (src/mm10_b.f:2343-3325); the local solve is mm10_solve
// (src/mm10_a.f:2860-3295) with 6 + 12 unknowns, the tangent mm10_tangent (:658-815) with
// ed = dgammadd = 0.  exact_j22 = 0 forms the Jacobian with the reference's formulas
// (sqrt(rho_F) in d h / d sigma and d h / d rho where mm10_h_mrr has sqrt(rho_P); no sign
// of tau on estress's c8 term; the fract > 1 branch of dgdt / dgdh drops terms), which
// slow the local Newton to linear convergence; exact_j22 = 1 differentiates the residual.
// One thread per voxel: the 18 x 18 Jacobian and its LU live in local memory.

constexpr int NH = 12;  // dislocation densities
constexpr bool ORNL = CPFFT_LAW == 4;

// the law's shear modulus: MRR's constant mu_0, ORNL's mu(T)
__device__ __forceinline__ double mrr_shear(const Crystal& s) {
  const CrysRec& c = *s.cr;
  return ORNL ? c.mu_0 - c.D_0 / (exp(c.T_0 / s.temp) - 1.0) : c.mu_0;
}
// ORNL: the attack frequency (exp(-G_0_y) when negative) and the slip exponent, 1 below
// the passing stress (fract < 0)
__device__ __forceinline__ double ornl_vs(const CrysRec& c) {
  return c.G_0_y < 0.0 ? exp(-c.G_0_y) : c.G_0_y;
}
__device__ __forceinline__ double mrr_pexp(const CrysRec& c, double fract) {
  return ORNL && fract < 0.0 ? 1.0 : c.p_v;
}
constexpr double MRR_PI = 3.141592653589793;
constexpr double MRR_NU = 0.3;  // Poisson's ratio of the dipole distance (mm10_h_mrr)

// the quantities of system a at (sigma, rho) every routine forms: resolved shear, forest
// and parallel densities, rate prefactor, passing and cutting stresses, the slip
// increment (mm10_slipinc_mrr, src/mm10_b.f:2477-2546) and, once per system, the pieces
// of its derivatives: slip / g0 and d slip / d fract (the reference's dgdt / dgdh
// evaluate the same exponential and powers again for every entry they fill; here the
// Jacobian's 288 d slip / d rho entries reuse each system's twelve values)
struct MrrSys {
  double rs, rhoF, rhoP, g0, tpass, tcut, fract, slip;
  double sg0;  // slip / g0 (exponential branch)
  double dsf;  // d slip / d fract (exponential branch)
  double m;    // slope of the linear extrapolation (fract > 1)
};

__device__ void mrr_sys(const Crystal& s, const double* st, const double* tt, int a, MrrSys& y) {
  const CrysRec& c = *s.cr;
  const double k = c.boltzman, th = s.temp, G = mrr_shear(s), b = c.burgers;
  y.rs = st[0] * s.ms[a][0] + st[1] * s.ms[a][1] + st[2] * s.ms[a][2] + st[3] * s.ms[a][3] +
         st[4] * s.ms[a][4] + st[5] * s.ms[a][5];
  double f = 0.0, p = 0.0;
  for (int q = 0; q < NH; q++) {
    f += __ldg(c.Gm + NH * a + q) * tt[q];
    p += __ldg(c.Hm + NH * a + q) * tt[q];
  }
  y.rhoF = f;
  y.rhoP = p;
  const double sp = sqrt(p);
  if (ORNL) {  // mobile density 0.1 rho_a, cutting stress tau_0 mu(T) / mu_0
    y.g0 = 0.1 * tt[a] * b * ornl_vs(c) / b * (c.u2 * b);
    y.tpass = c.u1 * G * b * sp;
    y.tcut = c.u3 * G / c.mu_0;
  } else {
    y.g0 = c.G_0_y * k * th / (c.u1 * c.u3 * G * b * b) * sp;
    y.tpass = c.u1 * G * b * sp;
    y.tcut = c.G_0_v / (c.u2 * c.u3 * b * b) * sqrt(f);
  }
  y.fract = (fabs(y.rs) - y.tpass) / y.tcut;
  const double Qk = c.G_0_v / k / th;
  y.sg0 = 0.0;
  y.dsf = 0.0;
  y.m = 0.0;
  if (y.fract > 1.0) {  // linear extrapolation past fract = 1
    y.m = y.g0 * (-c.q_v * Qk) * (-c.p_v) * sgn1(y.rs) / y.tcut;
    y.slip = s.tinc * (y.m * y.fract + y.g0);
  } else if (fabs(y.rs) > 0.0) {
    // exp(-Q / kT (1 - fract^p)^q) with the integral exponents of the usual parameters
    // (p = 1, q = 2) formed without pow
    const double pe = mrr_pexp(c, y.fract);
    const double fp = pe == 1.0 ? y.fract : pow(y.fract, pe);
    const double fp1 = pe == 1.0 ? 1.0 : pow(y.fract, pe - 1.0);
    const double base = 1.0 - fp;
    const double bq1 = c.q_v == 2.0 ? base : pow(base, c.q_v - 1.0);
    const double bq = c.q_v == 2.0 ? base * base : pow(base, c.q_v);
    y.sg0 = s.tinc * sgn1(y.rs) * exp(-Qk * bq);
    y.slip = y.sg0 * y.g0;
    y.dsf = y.slip * Qk * c.q_v * bq1 * pe * fp1;
  } else {
    y.slip = 0.0;
  }
}

// the twelve systems at one point
__device__ __forceinline__ void mrr_systems(const Crystal& s, const double* st, const double* tt,
                                            MrrSys* ys) {
  for (int a = 0; a < NH; a++) mrr_sys(s, st, tt, a, ys[a]);
}

// d slip / d rs (mm10_dgdt_mrr, src/mm10_b.f:3111-3198)
__device__ __forceinline__ double mrr_dgdt(const Crystal& s, const MrrSys& y) {
  const double dfract = sgn1(y.rs) / y.tcut;
  if (y.fract > 1.0) return s.cr->exact_j22 ? s.tinc * y.m * dfract : s.tinc * y.m;
  if (fabs(y.rs) > 0.0) return y.dsf * dfract;
  return 0.0;
}

// d slip_a / d rho_q (mm10_dgdh_mrr, src/mm10_b.f:3201-3306; ORNL: mm10_dgdh_ornl,
// :4224-4347, the prefactor depends on rho_a alone and the cutting stress on no density):
// g0, tau_pass and tau_cut scale with sqrt(rho_P) or sqrt(rho_F)
__device__ __forceinline__ double mrr_dgdh(const Crystal& s, const MrrSys& y, int a, int q) {
  const CrysRec& c = *s.cr;
  const double drhoF = __ldg(c.Gm + NH * a + q), drhoP = __ldg(c.Hm + NH * a + q);
  const double dg0 = ORNL ? (a == q ? 0.1 : 0.0) * c.burgers * ornl_vs(c) / c.burgers * (c.u2 * c.burgers)
                          : 0.5 * y.g0 * drhoP / y.rhoP;
  const double dtpass = 0.5 * y.tpass * drhoP / y.rhoP;
  const double dtcut = ORNL ? 0.0 : 0.5 * y.tcut * drhoF / y.rhoF;
  const double dfract = -(dtpass + y.fract * dtcut) / y.tcut;
  if (y.fract > 1.0) {
    const double Qk = c.G_0_v / c.boltzman / s.temp;
    const double K = (-c.q_v * Qk) * (-c.p_v) * sgn1(y.rs);
    const double dm = K * (dg0 / y.tcut - y.g0 * dtcut / (y.tcut * y.tcut));
    if (!c.exact_j22) return s.tinc * dm;
    return s.tinc * (dm * y.fract + y.m * dfract + dg0);
  }
  if (fabs(y.rs) > 0.0) return y.sg0 * dg0 + y.dsf * dfract;
  return 0.0;
}

// R1 (mm10_formR1, src/mm10_b.f:1061-1101): dbarp and wp of the systems' slips
__device__ void mrr_R1(const Crystal& s, const double* st, const MrrSys* ys, double* R1) {
  double dbar[6] = {0, 0, 0, 0, 0, 0}, w[3] = {0, 0, 0};
  for (int i = 0; i < NS; i++) {
    for (int a = 0; a < 6; a++) dbar[a] += ys[i].slip * s.ms[i][a];
    for (int a = 0; a < 3; a++) w[a] += ys[i].slip * s.qc[i][a];
  }
  double sw[6], wv1[6];
  symsw(st, w, sw);
  for (int a = 0; a < 6; a++) wv1[a] = s.D[a] - dbar[a];
  for (int a = 0; a < 6; a++) {
    double t = 0.0;
    for (int j = 0; j < 6; j++) t += Cv(s.C, a, j) * wv1[j];
    R1[a] = st[a] - s.nsig[a] - t + 2.0 * sw[a];
  }
}

__device__ void mrr_formR1(const Crystal& s, const double* st, const double* tt, double* R1) {
  MrrSys ys[NH];
  mrr_systems(s, st, tt, ys);
  mrr_R1(s, st, ys, R1);
}

// R = (R1, tt - h) (mm10_formR, mm10_h_mrr, src/mm10_b.f:1029-1047, 2549-2646); the
// densities' rates (h - rho_n) / tinc
__device__ void mrr_formR(const Crystal& s, const double* nrho, const double* x, double* R,
                          double* rate) {
  const CrysRec& c = *s.cr;
  const double* st = x;
  const double* tt = x + 6;
  MrrSys ys[NH];
  mrr_systems(s, st, tt, ys);
  mrr_R1(s, st, ys, R);
  const double k = c.boltzman, th = s.temp, G = mrr_shear(s), b = c.burgers;
  const double cdip = sqrt(3.0) * G * b / (16.0 * MRR_PI * (1.0 - MRR_NU));
  const double cM = (2.0 * k / (c.u1 * c.u2 * c.u3 * G * b * b * b)) * th;
  const double E = c.tau_hat_y * exp(-c.tau_a / k / th) / (k * th);
  for (int a = 0; a < NH; a++) {
    const MrrSys& y = ys[a];
    const double rho = tt[a], ars = fabs(y.rs);
    const double ddip = cdip / ars;
    const double rhoM = cM * sqrt(y.rhoF * y.rhoP);
    const double gd = fabs(y.slip / s.tinc);
    const double tem1 = c.u4 / b * sqrt(y.rhoP) * gd;
    const double tem2 = c.u6 * ddip / b * rhoM * gd;
    const double tem3 = c.u5 * rho * gd;
    const double tem4 = E * ars * rho * rho * pow(gd, c.tau_hat_v);
    const double h = nrho[a] + s.tinc * (tem1 + tem2 - tem3 - tem4);
    R[6 + a] = tt[a] - h;
    rate[a] = (h - nrho[a]) / s.tinc;
  }
}

// J11 (mm10_formJ11, src/mm10_b.f:177-257) with mm10_dgdt_mrr, ld = row stride of J
template <int ld>
__device__ void mrr_J11(const Crystal& s, const double* st, const MrrSys* ys, double* J) {
  for (int a = 0; a < 6; a++)
    for (int cc = 0; cc < 6; cc++) J[ld * a + cc] = 0.0;
  double w[3] = {0, 0, 0};
  for (int i = 0; i < NS; i++) {
    const double dg = mrr_dgdt(s, ys[i]);
    double sq[6];
    symsw(st, s.qc[i], sq);
    for (int a = 0; a < 6; a++) {
      const double wv = s.Cms[i][a] + 2.0 * sq[a];
      for (int cc = 0; cc < 6; cc++) J[ld * a + cc] += wv * (dg * s.ms[i][cc]);
    }
    for (int a = 0; a < 3; a++) w[a] += ys[i].slip * s.qc[i][a];
  }
  // mm10_iw (src/mm10_b.f:1590-1634) and the identity
  J[ld * 0 + 3] += 2.0 * w[2];  J[ld * 0 + 5] += -2.0 * w[1];
  J[ld * 1 + 3] += 2.0 * w[2];  J[ld * 1 + 4] += -2.0 * w[0];
  J[ld * 2 + 4] += 2.0 * w[0];  J[ld * 2 + 5] += 2.0 * w[1];
  J[ld * 3 + 0] += w[2];  J[ld * 3 + 1] += -w[2]; J[ld * 3 + 4] += -w[1]; J[ld * 3 + 5] += w[0];
  J[ld * 4 + 1] += w[0];  J[ld * 4 + 2] += -w[0]; J[ld * 4 + 3] += w[1];  J[ld * 4 + 5] += w[2];
  J[ld * 5 + 0] += w[1];  J[ld * 5 + 2] += -w[1]; J[ld * 5 + 3] += w[0];  J[ld * 5 + 4] += -w[2];
  for (int a = 0; a < 6; a++) J[ld * a + a] += 1.0;
}

// the 18 x 18 Jacobian (mm10_formJ, src/mm10_b.f:901-954), row-major: J12 (mm10_formJ12
// with mm10_dgdh_mrr), J21 = -estress (mm10_estress_mrr, :2859-2963), J22 = ehard
// (mm10_ehard_mrr, :2966-3092)
__device__ void mrr_formJ(const Crystal& s, const double* x, double* J) {
  constexpr int L = 6 + NH;
  const CrysRec& c = *s.cr;
  const double* st = x;
  const double* tt = x + 6;
  MrrSys ys[NH];
  mrr_systems(s, st, tt, ys);
  mrr_J11<L>(s, st, ys, J);
  for (int a = 0; a < 6; a++)
    for (int q = 0; q < NH; q++) J[L * a + 6 + q] = 0.0;
  const double k = c.boltzman, th = s.temp, G = mrr_shear(s), b = c.burgers;
  const double dt = s.tinc;
  const double cdip = sqrt(3.0) * G * b / (16.0 * MRR_PI * (1.0 - MRR_NU));
  const double cM = 2.0 * k / (c.u1 * c.u2 * c.u3 * G * b * b * b) * th;
  const double E = c.tau_hat_y * exp(-c.tau_a / k / th) / (k * th);
  const double c8 = c.tau_hat_v;
  for (int a = 0; a < NH; a++) {
    const MrrSys& y = ys[a];
    double dsh[NH];  // d slip_a / d rho_q
    for (int q = 0; q < NH; q++) dsh[q] = mrr_dgdh(s, y, a, q);
    // J12 column block of system a's slip
    {
      double sq[6];
      symsw(st, s.qc[a], sq);
      for (int q = 0; q < NH; q++)
        for (int r = 0; r < 6; r++) J[L * r + 6 + q] += (s.Cms[a][r] + 2.0 * sq[r]) * dsh[q];
    }
    const double rho = tt[a], sg = sgn1(y.rs), ars = fabs(y.rs);
    const double ddip = cdip / ars;
    const double dddip = -cdip / (ars * ars) * sg;
    const double rhoM = cM * sqrt(y.rhoF * y.rhoP);
    const double gd = fabs(y.slip / dt);
    const double dsl = mrr_dgdt(s, y) / dt;
    const double gdc8 = gd == 0.0 ? 0.0 : pow(gd, c8);   // gd^c8 (0 at gd = 0, c8 > 0)
    const double gdc81 = gd == 0.0 ? 0.0 : gdc8 / gd;     // gd^(c8 - 1), only where gd != 0
    double et;
    if (!c.exact_j22) {
      const double bad = gd == 0.0 ? 0.0 : c8 * ars * gdc81 * dsl;
      et = dt * (c.u4 / b * sqrt(y.rhoF) * sg * dsl + c.u6 / b * rhoM * (ddip * sg * dsl + dddip * gd) -
                 c.u5 * rho * sg * dsl - E * rho * rho * (bad + sg * gdc8));
    } else {
      const double dgd = sgn1(y.slip) * dsl;
      const double bad = gd == 0.0 ? 0.0 : c8 * ars * gdc81 * dgd;
      et = dt * (c.u4 / b * sqrt(y.rhoP) * dgd + c.u6 / b * rhoM * (ddip * dgd + dddip * gd) -
                 c.u5 * rho * dgd - E * rho * rho * (bad + sg * gdc8));
    }
    for (int r = 0; r < 6; r++) J[L * (6 + a) + r] = -et * s.ms[a][r];
    const double sqF = sqrt(y.rhoF), sqP = sqrt(y.rhoP), sqFP = sqrt(y.rhoF * y.rhoP);
    for (int q = 0; q < NH; q++) {
      const double drhoF = __ldg(c.Gm + NH * a + q), drhoP = __ldg(c.Hm + NH * a + q);
      const double drhoM = 0.5 * cM / sqFP * (drhoF * y.rhoP + y.rhoF * drhoP);
      const double d = a == q ? 1.0 : 0.0;
      const double dq = dsh[q] / dt;
      double e;
      if (!c.exact_j22) {
        const double bad = gd == 0.0 ? 0.0 : c8 * gdc81 * dq;
        e = d - dt * (c.u4 / b * (0.5 * drhoF / sqF * gd * sg + sqF * dq) +
                      c.u6 / b * (rhoM * ddip * dq + drhoM * ddip * gd * sg) -
                      c.u5 * (rho * dq + d * gd * sg) -
                      E * ars * (rho * rho * bad + 2.0 * rho * sg * d * gdc8)) * sg;
      } else {
        const double dgd = sgn1(y.slip) * dq;
        const double bad = gd == 0.0 ? 0.0 : c8 * gdc81 * dgd;
        e = d - dt * (c.u4 / b * (0.5 * drhoP / sqP * gd + sqP * dgd) +
                      c.u6 / b * ddip * (rhoM * dgd + drhoM * gd) - c.u5 * (rho * dgd + d * gd) -
                      E * ars * (rho * rho * bad + 2.0 * rho * d * gdc8));
      }
      J[L * (6 + a) + 6 + q] = e;
    }
  }
}

// mm10_solve (src/mm10_a.f:2860-3295) for 6 + 12 unknowns: the predictor's Newton on R1
// with the densities extrapolated along the previous step's rates, then the coupled
// Newton; Armijo line search c = 1e-4, halving, at most 11 trials.  Jl keeps the last
// Jacobian (mm10_tangent's).
__device__ bool mrr_solve(Crystal& cu, const double* nrho, const double* nrate, double dtinc,
                          double* stress, double* tt, double* Jl, bool& haveJ, int& iters,
                          int& piters, double* rate) {
  constexpr int L = 6 + NH;
  const CrysRec& c = *cu.cr;
  const double cls = 1.0e-4;
  double x[L];
  for (int i = 0; i < 6; i++) x[i] = stress[i];
  for (int i = 0; i < NH; i++) x[6 + i] = tt[i];
  double inR1;
  {  // ---- predict (:2975-3156)
    double d1[6], d2[6];
    for (int i = 0; i < 6; i++) { d1[i] = cu.D[i]; d2[i] = cu.nD[i]; }
    for (int k = 0; k < 2; k++) {
      double* d = k ? d2 : d1;
      const double dtr = (d[0] + d[1] + d[2]) / 3.0;
      d[0] -= dtr; d[1] -= dtr; d[2] -= dtr;
      const double t1 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      const double t2 = d[3] * d[3] + d[4] * d[4] + d[5] * d[5];
      if (t1 + t2 == 0.0) {
        for (int i = 0; i < 6; i++) d[i] = 0.0;
      } else {
        const double nn = sqrt(t1 + t2);
        for (int i = 0; i < 6; i++) d[i] = d[i] / nn;
      }
    }
    const double cos_ang = fmax(d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2] +
                                    (d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5]), 0.0);
    double x1[6], x2[NH], R1[6];
    for (int i = 0; i < 6; i++) x1[i] = x[i];
    for (int i = 0; i < NH; i++) x2[i] = x[6 + i] + cos_ang * nrate[i] * dtinc;
    mrr_formR1(cu, x1, x2, R1);
    double dot = 0;
    for (int a = 0; a < 6; a++) dot += R1[a] * R1[a];
    double nR1 = sqrt(dot);
    inR1 = nR1;
    int it = 0;
    while (nR1 > c.atol1 && nR1 / inR1 > c.rtol1) {
      double J[36], mJ[36], dx[6];
      {
        MrrSys ys[NH];
        mrr_systems(cu, x1, x2, ys);
        mrr_J11<6>(cu, x1, ys, J);
      }
      for (int a = 0; a < 36; a++) mJ[a] = -J[a];
      for (int a = 0; a < 6; a++) dx[a] = R1[a];
      lu_solve1<6>(mJ, dx);
      double ls1 = 0.5 * dot, ls2 = 0.0;
      for (int a = 0; a < 6; a++) {
        double wv = 0.0;
        for (int b = 0; b < 6; b++) wv += J[6 * b + a] * R1[b];
        ls2 += dx[a] * wv;
      }
      ls2 *= cls;
      double alpha = 1.0;
      for (int ls = 0;; ls++) {
        double xn[6];
        for (int a = 0; a < 6; a++) xn[a] = x1[a] + alpha * dx[a];
        mrr_formR1(cu, xn, x2, R1);
        dot = 0;
        for (int a = 0; a < 6; a++) dot += R1[a] * R1[a];
        nR1 = sqrt(dot);
        if (0.5 * dot <= ls1 + ls2 * alpha || ls > 10) {
          for (int a = 0; a < 6; a++) x1[a] = xn[a];
          break;
        }
        alpha *= 0.5;
      }
      it++;
      if (it > c.miter || anynan(x1, 6)) { piters += it; return false; }
    }
    piters += it;
    for (int i = 0; i < 6; i++) x[i] = x1[i];
    for (int i = 0; i < NH; i++) x[6 + i] = x2[i];
  }
  // ---- update (:3162-3293)
  double R[L];
  mrr_formR(cu, nrho, x, R, rate);
  double dot = 0;
  for (int a = 0; a < L; a++) dot += R[a] * R[a];
  double nR = sqrt(dot), inR = nR;
  if (inR == 0.0) inR = inR1;
  int it = 0;
  while ((nR > c.atol && nR / inR > c.rtol) || it < 1) {
    mrr_formJ(cu, x, Jl);
    haveJ = true;
    double mJ[L * L], dx[L];
    for (int a = 0; a < L * L; a++) mJ[a] = -Jl[a];
    for (int a = 0; a < L; a++) dx[a] = R[a];
    lu_solve1<L>(mJ, dx);
    double ls1 = 0.5 * dot, ls2 = 0.0;
    for (int a = 0; a < L; a++) {
      double wv = 0.0;
      for (int b = 0; b < L; b++) wv += Jl[L * b + a] * R[b];
      ls2 += dx[a] * wv;
    }
    ls2 *= cls;
    double alpha = 1.0;
    for (int ls = 0;; ls++) {
      double xn[L];
      for (int a = 0; a < L; a++) xn[a] = x[a] + alpha * dx[a];
      mrr_formR(cu, nrho, xn, R, rate);
      dot = 0;
      for (int a = 0; a < L; a++) dot += R[a] * R[a];
      nR = sqrt(dot);
      if (0.5 * dot <= ls1 + ls2 * alpha || ls > 10) {
        for (int a = 0; a < L; a++) x[a] = xn[a];
        break;
      }
      alpha *= 0.5;
    }
    it++;
    if (it > c.miter || anynan(x, L)) { iters += it; return false; }
  }
  iters += it;
  for (int i = 0; i < 6; i++) stress[i] = x[i];
  for (int i = 0; i < NH; i++) tt[i] = x[6 + i];
  return true;
}

// One voxel of an MRR grid: the material-point sequence of voxel_update (kinematics,
// mm10_solve_strup with sub-stepping, mm10_tangent, the rotation update, P and dP/dF)
// with the densities in history words H_RHO .. H_RHO + 23 (rates after the densities).
// The learned guess and the alternative starts do not apply: every implicit solve
// starts from the reference's predictor.
__device__ void voxel_update_mrr(const StressArgs& a, long long v, int& iters, int& piters,
                                 bool& ok) {
  constexpr int L = 6 + NH;
  const long long N3 = a.N3;
  double Fn[9], Fn1[9];
  for (int i = 0; i < 9; i++) {
    Fn[i] = __ldg(a.Fn + i * N3 + v);
    Fn1[i] = __ldg(a.Fn1 + i * N3 + v);
  }
  const OriRec* rec = a.oris + __ldg(a.ori + v);
  const CrysRec* cr = a.cryss + __ldg(a.crys + v);
  // history at n (step 1: mm10_init_mrr, src/mm10_a.f:2205-2223)
  double nsig[6], nRp[9], nD[6], nrho[NH], nrate[NH];
  if (a.step == 1) {
    for (int i = 0; i < 6; i++) { nsig[i] = 0.0; nD[i] = 0.0; }
    const double r0 = cr->theta_0 == 0.0 ? 1.0e8 : cr->theta_0;
    for (int i = 0; i < NH; i++) { nrho[i] = r0; nrate[i] = 0.0; }
    for (int i = 0; i < 9; i++) nRp[i] = (i % 4 == 0) ? 1.0 : 0.0;
  } else {
    for (int i = 0; i < 6; i++) nsig[i] = a.hist_n[(H_SIG + i) * N3 + v];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) nRp[3 * i + j] = a.hist_n[(H_RP + 3 * j + i) * N3 + v];
    for (int i = 0; i < 6; i++) nD[i] = a.hist_n[(H_D + i) * N3 + v];
    for (int i = 0; i < NH; i++) {
      nrho[i] = a.hist_n[(H_RHO + i) * N3 + v];
      nrate[i] = a.hist_n[(H_RHO + NH + i) * N3 + v];
    }
  }
  double rnh[9], rn1[9], fnhinv[9], uddt[6];
  kinematics(Fn, Fn1, rnh, rn1, fnhinv, uddt);
  Crystal s;
  s.cr = cr;
  s.C = rec->C;
  s.nsig = nsig;
  for (int i = 0; i < 6; i++) s.nD[i] = nD[i];
  setup_np1(s, rec, uddt, a.dt, rn1, nRp);
  s.temp = TEMP;
  double stress[6], tt[NH], rate[NH];
  for (int i = 0; i < 6; i++) stress[i] = nsig[i];
  for (int i = 0; i < NH; i++) { tt[i] = nrho[i]; rate[i] = 0.0; }
  double t1 = 0, t2 = 0;
  for (int i = 0; i < 6; i++) { t1 += uddt[i] * uddt[i]; t2 += stress[i] * stress[i]; }
  const bool no_load = t1 == 0.0 && t2 == 0.0;
  const bool iter0 = a.iter == 0;
  double cep[36];
  double Jl[L * L];
  bool haveJ = false;
  ok = true;
  if (iter0 || no_load) {  // mm10_solve_strup_a (src/mm10_a.f:2721-2743)
    for (int i = 0; i < 36; i++) cep[i] = __ldg(rec->C + i);
    if (!no_load) {
      double R1[6];
      mrr_formR1(s, stress, tt, R1);
      for (int i = 0; i < 6; i++) stress[i] -= R1[i];
    }
  } else {  // mm10_solve_strup_iterate (:2747-2843): at most 4 halvings
    double ostress[6], ott[NH], frac = 0.0, stp = 1.0;
    for (int i = 0; i < 6; i++) ostress[i] = stress[i];
    for (int i = 0; i < NH; i++) ott[i] = tt[i];
    int cuts = 0;
    bool fail = false;
    while (frac < 1.0) {
      s.tinc = a.dt * (stp + frac);
      for (int i = 0; i < 6; i++) s.D[i] = uddt[i] * (stp + frac);
      s.temp = TEMP * (stp + frac);  // n's temperature is zero (:2769)
      for (int i = 0; i < NH; i++) tt[i] = nrho[i];
      double rsub[NH];
      fail = !mrr_solve(s, nrho, nrate, a.dt * stp, stress, tt, Jl, haveJ, iters, piters, rsub);
      if (fail) {
        for (int i = 0; i < 6; i++) stress[i] = ostress[i];
        for (int i = 0; i < NH; i++) tt[i] = ott[i];
        stp *= 0.5;
        if (++cuts > 4) break;
        fail = false;
      } else {
        for (int i = 0; i < 6; i++) ostress[i] = stress[i];
        for (int i = 0; i < NH; i++) { ott[i] = tt[i]; rate[i] = rsub[i]; }
        frac += stp;
      }
    }
    if (cuts && a.stats) atomicAdd(a.stats + 4, 1ull);
    s.tinc = a.dt;
    for (int i = 0; i < 6; i++) s.D[i] = uddt[i];
    s.temp = TEMP;
    ok = !(fail || anynan(stress, 6) || anynan(tt, NH));
    if (ok) {
      // mm10_tangent (:658-815), ed = dgammadd = 0: T = (J11 - J12 J22^-1 J21)^-1 C
      double A22[NH * NH], B[NH * 6];
      for (int r = 0; r < NH; r++)
        for (int q = 0; q < NH; q++) A22[NH * r + q] = Jl[L * (6 + r) + 6 + q];
      // LU of J22 once, then the six columns of J21
      int piv[NH];
      for (int k = 0; k < NH; k++) {
        int p = k;
        double best = fabs(A22[NH * k + k]);
        for (int i = k + 1; i < NH; i++)
          if (fabs(A22[NH * i + k]) > best) { best = fabs(A22[NH * i + k]); p = i; }
        piv[k] = p;
        if (p != k)
          for (int j = 0; j < NH; j++) { double t = A22[NH * k + j]; A22[NH * k + j] = A22[NH * p + j]; A22[NH * p + j] = t; }
        const double inv = 1.0 / A22[NH * k + k];
        for (int i = k + 1; i < NH; i++) {
          const double l = A22[NH * i + k] * inv;
          A22[NH * i + k] = l;
          for (int j = k + 1; j < NH; j++) A22[NH * i + j] -= l * A22[NH * k + j];
        }
      }
      for (int col = 0; col < 6; col++) {
        double bcol[NH];
        for (int r = 0; r < NH; r++) bcol[r] = Jl[L * (6 + r) + col];
        for (int k = 0; k < NH; k++)
          if (piv[k] != k) { double t = bcol[k]; bcol[k] = bcol[piv[k]]; bcol[piv[k]] = t; }
        for (int i = 1; i < NH; i++)
          for (int k = 0; k < i; k++) bcol[i] -= A22[NH * i + k] * bcol[k];
        for (int i = NH - 1; i >= 0; i--) {
          double acc = bcol[i];
          for (int k = i + 1; k < NH; k++) acc -= A22[NH * i + k] * bcol[k];
          bcol[i] = acc / A22[NH * i + i];
        }
        for (int r = 0; r < NH; r++) B[6 * r + col] = bcol[r];
      }
      double JJ[36], T[36];
      for (int r = 0; r < 6; r++)
        for (int col = 0; col < 6; col++) {
          double acc = Jl[L * r + col];
          for (int q = 0; q < NH; q++) acc -= Jl[L * r + 6 + q] * B[6 * q + col];
          JJ[6 * r + col] = acc;
        }
      for (int col = 0; col < 6; col++) {
        double m[36], bb[6];
        for (int i = 0; i < 36; i++) m[i] = JJ[i];
        for (int i = 0; i < 6; i++) bb[i] = __ldg(rec->C + 6 * i + col);
        lu_solve1<6>(m, bb);
        for (int i = 0; i < 6; i++) T[6 * i + col] = bb[i];
      }
      for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) cep[6 * i + j] = (T[6 * i + j] + T[6 * j + i]) * 0.5;
    } else {
      for (int i = 0; i < 6; i++) stress[i] = nsig[i];
      for (int i = 0; i < NH; i++) { tt[i] = nrho[i]; rate[i] = 0.0; }
      for (int i = 0; i < 36; i++) cep[i] = __ldg(rec->C + i);
    }
  }
  // ---- plastic rotation (mm10_update_rotation, src/mm10_a.f:3310-3327)
  double Rp[9];
  if (!ok) {
    for (int i = 0; i < 9; i++) Rp[i] = nRp[i];
  } else if (iter0 || no_load) {
    for (int i = 0; i < 9; i++) Rp[i] = 0.0;
  } else {
    double tr[9], RW[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) tr[3 * i + j] = nRp[3 * j + i];
    rt2rvw(tr, RW);
    double wb[3] = {0, 0, 0};
    for (int i = 0; i < NS; i++) {
      MrrSys y;
      mrr_sys(s, stress, tt, i, y);
      double q0[3], qs[3];
      for (int k = 0; k < 3; k++) q0[k] = __ldg(rec->qs + 3 * i + k);
      for (int k = 0; k < 3; k++) qs[k] = RW[3 * k] * q0[0] + RW[3 * k + 1] * q0[1] + RW[3 * k + 2] * q0[2];
      for (int k = 0; k < 3; k++) wb[k] += y.slip * qs[k];
    }
    double W[9] = {0.0, wb[2], wb[1], -wb[2], 0.0, wb[0], -wb[1], -wb[0], 0.0};
    const double al = sqrt(W[5] * W[5] + W[2] * W[2] + W[1] * W[1]);
    double ex[9];
    if (al < 1.0e-16) {
      for (int i = 0; i < 9; i++) ex[i] = 0.0;
    } else {
      double WW[9];
      mm3(W, W, WW);
      const double ca = (1.0 - cos(al)) / (al * al), sa = sin(al) / al;
      for (int i = 0; i < 9; i++) ex[i] = ca * WW[i] + sa * W[i];
    }
    ex[0] += 1.0; ex[4] += 1.0; ex[8] += 1.0;
    mm3(ex, nRp, Rp);
  }
  // ---- history n+1
  for (int i = 0; i < 6; i++) a.hist_np1[(H_SIG + i) * N3 + v] = stress[i];
  a.hist_np1[H_TT * N3 + v] = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a.hist_np1[(H_RP + 3 * j + i) * N3 + v] = Rp[3 * i + j];
  for (int i = 0; i < 6; i++) a.hist_np1[(H_D + i) * N3 + v] = uddt[i];
  a.hist_np1[H_TTR * N3 + v] = 0.0;
  a.hist_np1[H_U * N3 + v] = 0.0;
  a.hist_np1[(H_U + 1) * N3 + v] = 0.0;
  for (int i = 0; i < 6; i++)
    a.hist_np1[(H_EPS + i) * N3 + v] = (a.step == 1 ? 0.0 : a.hist_n[(H_EPS + i) * N3 + v]) + uddt[i];
  for (int i = 0; i < NH; i++) {
    a.hist_np1[(H_RHO + i) * N3 + v] = tt[i];
    a.hist_np1[(H_RHO + NH + i) * N3 + v] = rate[i];
  }
  store_P_K4(a, v, Fn, Fn1, stress, cep, rnh, rn1, fnhinv);
}
