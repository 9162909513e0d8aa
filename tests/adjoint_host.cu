// Host build of the adjoint's per-pair and per-body functions (test infrastructure only).
//
// The adjoint's geometry, law and integrator are __host__ __device__ templates; this file runs
// them on the host, one pair or body after another, over a whole window (every state kept, no
// checkpoints), so that the CPU test suite can check the reverse pass against central
// differences of the oracle's frozen-pair window without a GPU.  The product path is the CUDA
// kernels of sqdem_adjoint.cu; nothing here is loaded by the package.
#include "../sudodem_gb300/csrc/sqdem_adjoint.cu"
#include <cmath>
// r_max of Superquadrics::Initial (Superquadrics.cpp:47-93); the library's version lives in the
// engine's translation unit
extern "C" sqdem_status sqdem_shape_props(double rx, double ry, double rz, double e1, double e2, double* out5) {
  double r = rx > ry ? rx : ry; r = r > rz ? r : rz;
  if (e1 < 1.0 || e2 < 1.0) r *= std::pow(2.0, 0.5);
  out5[0] = out5[1] = out5[2] = out5[3] = 0; out5[4] = r;
  return SQDEM_OK;
}
// branch tape of the host window (sqdem_adj_set_branches' modes), kept between runs
static int g_brMode = BR_OFF, g_brSteps = 0;
static std::vector<unsigned> g_brPair, g_brBody;
static double g_brReport[5] = {0, 0, 0, 0, 0};
extern "C" int adjh_set_branches(int mode) {
  if (mode < BR_OFF || mode > BR_FORCE || (mode == BR_FORCE && g_brSteps == 0)) return 1;
  g_brMode = mode;
  return 0;
}
extern "C" void adjh_branch_report(double* out5) { for (int k = 0; k < 5; k++) out5[k] = g_brReport[k]; }
extern "C" double adjh_run(int n, const int* kind, const double* shape5, const int* was, const int* mat,
                           const double* state37, long npairs, const double* intr57, double dt, const double* g3,
                           double damping, int nmat, const double* Kn, const double* Ks, const double* fa,
                           const double* eps2, int nsteps, const double* wF3, const double* wX3, double* gEps,
                           double* gKn, double* gKs, double* gMu, double* fin16, unsigned long long* sigOut,
                           long long* mism) {
  sqdem_adj A0; sqdem_adj* a = &A0;
  a->nb = n; a->dt = dt; a->damping = damping; for (int k = 0; k < 3; k++) a->g[k] = g3[k];
  a->kind.assign(kind, kind + n); a->mat.assign(mat, mat + n);
  a->Kn.assign(Kn, Kn + nmat); a->Ks.assign(Ks, Ks + nmat); a->fa.assign(fa, fa + nmat); a->nmat = nmat;
  std::vector<int> hFlag; std::vector<double> hDepth; std::vector<double2> hAng; std::vector<double4> hN, hS;
  for (long r = 0; r < npairs; r++) {
    const double* o = intr57 + r * 57;
    int i1 = (int)o[0], i2 = (int)o[1];
    if (kind[i1] == 1 && kind[i2] == 1) continue;
    if (kind[i1] == 0 && kind[i2] == 1) std::swap(i1, i2);
    a->ids.push_back(make_int2(i1, i2));
    hFlag.push_back(o[3] != 0 ? CF_GEOM : 0); hDepth.push_back(o[4]); hAng.push_back(make_double2(o[5], o[6]));
    hN.push_back(make_double4(o[10], o[11], o[12], 0)); hS.push_back(make_double4(o[29], o[30], o[31], 0));
  }
  const int P = a->P = (int)a->ids.size();
  std::vector<int> cntB(n + 1, 0), start(n + 1, 0), list(2 * (size_t)P + 1);
  for (int c = 0; c < P; c++) { cntB[a->ids[c].x]++; cntB[a->ids[c].y]++; }
  for (int i = 0; i < n; i++) start[i + 1] = start[i] + cntB[i];
  std::vector<int> fill(start.begin(), start.end() - 1);
  for (int c = 0; c < P; c++) { list[fill[a->ids[c].x]++] = 2 * c; list[fill[a->ids[c].y]++] = 2 * c + 1; }
  std::vector<double4> hShp(n), hMI(n), ph(P + 1); std::vector<double2> hEps(n); std::vector<int4> hInfo(n);
  for (int i = 0; i < n; i++) {
    const double* s5 = shape5 + i * 5; const double* s = state37 + i * 37;
    double props[5] = {0, 0, 0, 0, 0};
    if (kind[i] == 0) sqdem_shape_props(s5[0], s5[1], s5[2], s5[3], s5[4], props);
    hShp[i] = make_double4(s5[0], s5[1], s5[2], props[4]);
    hEps[i] = make_double2(eps2[2 * i], eps2[2 * i + 1]);
    hMI[i] = make_double4(s[33], s[34], s[35], s[36]);
    hInfo[i] = make_int4(kind[i], was[2 * i], was[2 * i + 1], 0);
  }
  for (int c = 0; c < P; c++) { double kn, ks, t; physOf(a, c, kn, ks, t); ph[c] = make_double4(kn, ks, t, 0); }
  unsigned long long cnt[A_NCOUNT] = {};
  Consts C; C.nb = n; C.P = P; C.dt = dt; for (int k = 0; k < 3; k++) C.g[k] = g3[k]; C.damping = damping;
  C.shp = hShp.data(); C.eps = hEps.data(); C.massI = hMI.data(); C.binfo = hInfo.data(); C.ids = a->ids.data();
  C.phys = ph.data(); C.bStart = start.data(); C.bList = list.data(); C.cnt = cnt;
  if (g_brMode == BR_FORCE && nsteps > g_brSteps) return NAN;
  if (g_brMode == BR_RECORD) {
    g_brPair.assign((size_t)nsteps * P * BR_WORDS + 1, 0u);
    g_brBody.assign((size_t)nsteps * n, 0u);
    g_brSteps = nsteps;
  }
  C.brMode = g_brMode; C.brPair = g_brPair.data(); C.brBody = g_brBody.data();
  StateLayout L; L.init(n, P);
  std::vector<std::vector<char>> st(nsteps + 1, std::vector<char>(L.bytes, 0));
  {
    State hv = L.view(st[0].data());
    for (int i = 0; i < n; i++) {
      const double* s = state37 + i * 37;
      hv.pos[i] = make_double4(s[0], s[1], s[2], 0); hv.ori[i] = make_double4(s[3], s[4], s[5], s[6]);
      hv.vel[i] = make_double4(s[7], s[8], s[9], 0); hv.angVel[i] = make_double4(s[10], s[11], s[12], 0);
      hv.angMom[i] = make_double4(s[13], s[14], s[15], 0);
    }
    for (int c = 0; c < P; c++) { hv.flag[c] = hFlag[c]; hv.depth[c] = hDepth[c]; hv.angle[c] = hAng[c]; hv.normal[c] = hN[c]; hv.shear[c] = hS[c]; }
  }
  std::vector<std::vector<double4>> Fv(nsteps, std::vector<double4>(P + 1)), Cp(nsteps, std::vector<double4>(P + 1));
  std::vector<std::vector<int>> Code(nsteps, std::vector<int>(P + 1));
  for (int t = 0; t < nsteps; t++) {
    st[t + 1] = st[t];
    State S = L.view(st[t + 1].data());
    StepOut O; O.Fv = Fv[t].data(); O.cp = Cp[t].data(); O.code = Code[t].data();
    for (int c = 0; c < P; c++) fwdContact(C, S, O, t, c);
    for (int b = 0; b < n; b++) fwdBody(C, S, O, t, b);
  }
  // loss
  std::vector<double4> wF(n), wX(n);
  for (int i = 0; i < n; i++) {
    wF[i] = wF3 ? make_double4(wF3[3 * i], wF3[3 * i + 1], wF3[3 * i + 2], 0) : make_double4(0, 0, 0, 0);
    wX[i] = wX3 ? make_double4(wX3[3 * i], wX3[3 * i + 1], wX3[3 * i + 2], 0) : make_double4(0, 0, 0, 0);
  }
  double loss = 0;
  {
    State S = L.view(st[nsteps].data());
    StepOut O; O.Fv = Fv[nsteps - 1].data(); O.cp = Cp[nsteps - 1].data(); O.code = Code[nsteps - 1].data();
    for (int b = 0; b < n; b++) {
      V3<double> f, m; const V3<double> pos = xyz(S.pos[b]);
      gatherFT(C, O, b, pos, f, m);
      loss += dot(xyz(wF[b]), f) + dot(xyz(wX[b]), pos);
    }
    for (int i = 0; i < n; i++) {
      double* o = fin16 + i * 16; const double4 p = S.pos[i], q = S.ori[i], v = S.vel[i], w = S.angVel[i], Lm = S.angMom[i];
      o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
      o[7] = v.x; o[8] = v.y; o[9] = v.z; o[10] = w.x; o[11] = w.y; o[12] = w.z; o[13] = Lm.x; o[14] = Lm.y; o[15] = Lm.z;
    }
  }
  sigOut[0] = cnt[A_SIG] + cnt[A_SIGB];
  g_brReport[0] = (double)cnt[A_BRDEC]; g_brReport[1] = (double)cnt[A_BRDIS]; g_brReport[2] = (double)cnt[A_BRUNF];
  g_brReport[3] = g_brSteps; g_brReport[4] = (double)cnt[A_BRCUSP];
  C.brMode = BR_OFF;   // the reverse pass evaluates its decisions
  // backward
  std::vector<double4> lPos(wX), lOri(n), lVel(n), lW(n), lL(n), lF(n), lT(n), lN(P + 1), lS(P + 1), con(8 * (size_t)P + 8),
      accE(P + 1), accP(P + 1);
  std::vector<double2> lAng(P + 1);
  for (auto* v : {&lOri, &lVel, &lW, &lL, &lF, &lT}) for (auto& x : *v) x = make_double4(0, 0, 0, 0);
  for (auto* v : {&lN, &lS, &accE, &accP}) for (auto& x : *v) x = make_double4(0, 0, 0, 0);
  for (auto& x : lAng) x = make_double2(0, 0);
  Adj A; A.lPos = lPos.data(); A.lOri = lOri.data(); A.lVel = lVel.data(); A.lW = lW.data(); A.lL = lL.data();
  A.lF = lF.data(); A.lT = lT.data(); A.lAng = lAng.data(); A.lN = lN.data(); A.lS = lS.data(); A.con = con.data();
  A.accEps = accE.data(); A.accPhys = accP.data(); A.wF = wF.data(); A.wX = wX.data();
  for (int t = nsteps - 1; t >= 0; t--) {
    State S = L.view(st[t].data());
    StepOut O; O.Fv = Fv[t].data(); O.cp = Cp[t].data(); O.code = Code[t].data();
    for (int b = 0; b < n; b++) bwdBody(C, S, O, A, t == nsteps - 1, b);
    for (int c = 0; c < P; c++) bwdContact(C, S, O, A, c);
    for (int b = 0; b < n; b++) bwdGather(C, A, b);
  }
  *mism = (long long)cnt[A_MISMATCH];
  for (int i = 0; i < 2 * n; i++) gEps[i] = 0;
  for (int m = 0; m < nmat; m++) gKn[m] = gKs[m] = gMu[m] = 0;
  for (int c = 0; c < P; c++) {
    const int id1 = a->ids[c].x, id2 = a->ids[c].y;
    if (kind[id1] == 0) { gEps[2 * id1] += accE[c].x; gEps[2 * id1 + 1] += accE[c].y; }
    gEps[2 * id2] += accE[c].z; gEps[2 * id2 + 1] += accE[c].w;
    const int m1 = mat[id1], m2 = mat[id2];
    if (id1 > 5) {
      const double s1 = Kn[m1] + Kn[m2], t1 = Ks[m1] + Ks[m2];
      gKn[m1] += accP[c].x * 2.0 * Kn[m2] * Kn[m2] / (s1 * s1); gKn[m2] += accP[c].x * 2.0 * Kn[m1] * Kn[m1] / (s1 * s1);
      gKs[m1] += accP[c].y * 2.0 * Ks[m2] * Ks[m2] / (t1 * t1); gKs[m2] += accP[c].y * 2.0 * Ks[m1] * Ks[m1] / (t1 * t1);
      gMu[(fa[m2] < fa[m1]) ? m2 : m1] += accP[c].z;
    } else { gKn[m1] += accP[c].x; gKs[m1] += accP[c].y; gMu[m1] += accP[c].z; }
  }
  return loss;
}
