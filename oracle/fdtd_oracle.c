/*
 * fdtd_oracle.c — ORACLE (test infrastructure only): a plain C restatement of gprMax v3.1.7's
 * CPU field-update kernels, used as the checker of the GPU solver. Nothing in the product path
 * links or calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg do.
 *
 * Each function follows the loops, index ranges and expression order of the reference:
 *   oracle_update_electric       gprMax/fields_updates_ext.pyx:30-110   (update_electric)
 *   oracle_update_magnetic       gprMax/fields_updates_ext.pyx:352-412  (update_magnetic)
 *   oracle_update_dispersive_A   gprMax/fields_updates_ext.pyx:113-181 and :238-297
 *   oracle_update_dispersive_B   gprMax/fields_updates_ext.pyx:183-236 and :299-349
 *   oracle_pml_electric          gprMax/pml_updates/pml_updates_electric_{HORIPML,MRIPML}_ext.pyx
 *                                (12 functions each: order{1,2}_{x,y,z}{minus,plus})
 *   oracle_pml_magnetic          gprMax/pml_updates/pml_updates_magnetic_{HORIPML,MRIPML}_ext.pyx
 * The 48 slab functions are written once, parameterised by direction; the per-direction
 * field components, signs, stencils and profile indexing are those of the reference files
 * (e.g. electric HORIPML order1_xminus :26-88, order2_xminus :89-158, order1_zminus :562-624;
 * magnetic HORIPML order1_xminus :26-88; MRIPML electric order1_xminus :26-89, order2 :91-162).
 *
 * Arrays use the reference's shapes and C order: fields [nx+1][ny+1][nz+1] fp32, ID
 * [6][nx+1][ny+1][nz+1] uint32, dispersive T [P][nx+1][ny+1][nz+1] complex64 (real pairs),
 * coefficients [nmat][5] fp32 and [nmat][3P] complex64, Phi [order][n1][n2][n3] fp32.
 * Built with -ffp-contract=off so every product and sum is rounded as written.
 *
 * `real` is float (the reference's default fp32 build, constants.pxd floattype_t). Compiled
 * with -DORACLE_F64 it is double and the complex state is double pairs: the same loops in
 * fp64, the "fp64 run of the same grid" that fp32 results are measured against.
 */
#include <stdint.h>
#include <stddef.h>

#ifdef ORACLE_F64
typedef double real;
#else
typedef float real;
#endif

#define IDX(i, j, k) (((size_t)(i) * NY + (j)) * NZ + (k))

/* electric update, standard materials: fields_updates_ext.pyx:30-110 */
void oracle_update_electric(int nx, int ny, int nz, const real* cE, const uint32_t* ID,
                            real* Ex, real* Ey, real* Ez,
                            const real* Hx, const real* Hy, const real* Hz) {
  const size_t NY = ny + 1, NZ = nz + 1, NC = (size_t)(nx + 1) * NY * NZ;
  const uint32_t *IDx = ID, *IDy = ID + NC, *IDz = ID + 2 * NC;
  int i, j, k;
  if (nx == 1) {
    for (i = 0; i < nx; i++) for (j = 1; j < ny; j++) for (k = 1; k < nz; k++) {
      const real* c = cE + 5 * (size_t)IDx[IDX(i, j, k)];
      Ex[IDX(i, j, k)] = c[0] * Ex[IDX(i, j, k)] + c[2] * (Hz[IDX(i, j, k)] - Hz[IDX(i, j - 1, k)]) - c[3] * (Hy[IDX(i, j, k)] - Hy[IDX(i, j, k - 1)]);
    }
  } else if (ny == 1) {
    for (i = 1; i < nx; i++) for (j = 0; j < ny; j++) for (k = 1; k < nz; k++) {
      const real* c = cE + 5 * (size_t)IDy[IDX(i, j, k)];
      Ey[IDX(i, j, k)] = c[0] * Ey[IDX(i, j, k)] + c[3] * (Hx[IDX(i, j, k)] - Hx[IDX(i, j, k - 1)]) - c[1] * (Hz[IDX(i, j, k)] - Hz[IDX(i - 1, j, k)]);
    }
  } else if (nz == 1) {
    for (i = 1; i < nx; i++) for (j = 1; j < ny; j++) for (k = 0; k < nz; k++) {
      const real* c = cE + 5 * (size_t)IDz[IDX(i, j, k)];
      Ez[IDX(i, j, k)] = c[0] * Ez[IDX(i, j, k)] + c[1] * (Hy[IDX(i, j, k)] - Hy[IDX(i - 1, j, k)]) - c[2] * (Hx[IDX(i, j, k)] - Hx[IDX(i, j - 1, k)]);
    }
  } else {
#pragma omp parallel for private(j, k) schedule(static)
    for (i = 1; i < nx; i++) for (j = 1; j < ny; j++) for (k = 1; k < nz; k++) {
      const real* a = cE + 5 * (size_t)IDx[IDX(i, j, k)];
      const real* b = cE + 5 * (size_t)IDy[IDX(i, j, k)];
      const real* c = cE + 5 * (size_t)IDz[IDX(i, j, k)];
      Ex[IDX(i, j, k)] = a[0] * Ex[IDX(i, j, k)] + a[2] * (Hz[IDX(i, j, k)] - Hz[IDX(i, j - 1, k)]) - a[3] * (Hy[IDX(i, j, k)] - Hy[IDX(i, j, k - 1)]);
      Ey[IDX(i, j, k)] = b[0] * Ey[IDX(i, j, k)] + b[3] * (Hx[IDX(i, j, k)] - Hx[IDX(i, j, k - 1)]) - b[1] * (Hz[IDX(i, j, k)] - Hz[IDX(i - 1, j, k)]);
      Ez[IDX(i, j, k)] = c[0] * Ez[IDX(i, j, k)] + c[1] * (Hy[IDX(i, j, k)] - Hy[IDX(i - 1, j, k)]) - c[2] * (Hx[IDX(i, j, k)] - Hx[IDX(i, j - 1, k)]);
    }
    /* Ex at i = 0 */
    for (j = 1; j < ny; j++) for (k = 1; k < nz; k++) {
      const real* a = cE + 5 * (size_t)IDx[IDX(0, j, k)];
      Ex[IDX(0, j, k)] = a[0] * Ex[IDX(0, j, k)] + a[2] * (Hz[IDX(0, j, k)] - Hz[IDX(0, j - 1, k)]) - a[3] * (Hy[IDX(0, j, k)] - Hy[IDX(0, j, k - 1)]);
    }
    /* Ey at j = 0 */
    for (i = 1; i < nx; i++) for (k = 1; k < nz; k++) {
      const real* b = cE + 5 * (size_t)IDy[IDX(i, 0, k)];
      Ey[IDX(i, 0, k)] = b[0] * Ey[IDX(i, 0, k)] + b[3] * (Hx[IDX(i, 0, k)] - Hx[IDX(i, 0, k - 1)]) - b[1] * (Hz[IDX(i, 0, k)] - Hz[IDX(i - 1, 0, k)]);
    }
    /* Ez at k = 0 */
    for (i = 1; i < nx; i++) for (j = 1; j < ny; j++) {
      const real* c = cE + 5 * (size_t)IDz[IDX(i, j, 0)];
      Ez[IDX(i, j, 0)] = c[0] * Ez[IDX(i, j, 0)] + c[1] * (Hy[IDX(i, j, 0)] - Hy[IDX(i - 1, j, 0)]) - c[2] * (Hx[IDX(i, j, 0)] - Hx[IDX(i, j - 1, 0)]);
    }
  }
}

/* complex helpers (complex64 stored as real pairs) */
typedef struct { real re, im; } cf;
static inline cf cmul(cf a, cf b) { cf r; r.re = a.re * b.re - a.im * b.im; r.im = a.re * b.im + a.im * b.re; return r; }
static inline cf cscale(cf a, real x) { cf r; r.re = a.re * x; r.im = a.im * x; return r; }
static inline cf cadd(cf a, cf b) { cf r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static inline cf csub(cf a, cf b) { cf r; r.re = a.re - b.re; r.im = a.im - b.im; return r; }

/* dispersive part A for one component: phi = sum Re(c0) Re(T); T = c1 T + c2 E; E update - srce*phi
 * (fields_updates_ext.pyx:113-181 multipole, :238-297 one pole) */
static void disp_A_comp(int comp, int i0, int i1, int j0, int j1, int k0, int k1, int nx, int ny, int nz,
                        int P, const real* cE, const cf* cD, const uint32_t* IDc, cf* T, real* F,
                        const real* Ha, const real* Hb, int da_i, int da_j, int da_k,
                        int db_i, int db_j, int db_k, int ca, int cb) {
  const size_t NY = ny + 1, NZ = nz + 1, NC = (size_t)(nx + 1) * NY * NZ;
  int i, j, k, p;
  (void)comp;
#pragma omp parallel for private(j, k, p) schedule(static)
  for (i = i0; i < i1; i++) for (j = j0; j < j1; j++) for (k = k0; k < k1; k++) {
    const size_t q = IDX(i, j, k);
    const uint32_t m = IDc[q];
    const real* c = cE + 5 * (size_t)m;
    const cf* d = cD + 3 * (size_t)P * m;
    real phi = 0;
    for (p = 0; p < P; p++) {
      cf t = T[p * NC + q];
      phi = phi + d[3 * p].re * t.re;
      T[p * NC + q] = cadd(cmul(d[3 * p + 1], t), cscale(d[3 * p + 2], F[q]));
    }
    F[q] = c[0] * F[q] + c[ca] * (Ha[q] - Ha[IDX(i - da_i, j - da_j, k - da_k)]) - c[cb] * (Hb[q] - Hb[IDX(i - db_i, j - db_j, k - db_k)]) - c[4] * phi;
  }
}

void oracle_update_dispersive_A(int nx, int ny, int nz, int P, const real* cE, const real* cDf,
                                const uint32_t* ID, real* Txf, real* Tyf, real* Tzf,
                                real* Ex, real* Ey, real* Ez,
                                const real* Hx, const real* Hy, const real* Hz) {
  const size_t NC = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  const cf* cD = (const cf*)cDf;
  if (ny != 1 || nz != 1)  /* Ex: CBy*(Hz - Hz[j-1]) - CBz*(Hy - Hy[k-1]) */
    disp_A_comp(0, 0, nx, 1, ny, 1, nz, nx, ny, nz, P, cE, cD, ID, (cf*)Txf, Ex, Hz, Hy, 0, 1, 0, 0, 0, 1, 2, 3);
  if (nx != 1 || nz != 1)  /* Ey: CBz*(Hx - Hx[k-1]) - CBx*(Hz - Hz[i-1]) */
    disp_A_comp(1, 1, nx, 0, ny, 1, nz, nx, ny, nz, P, cE, cD, ID + NC, (cf*)Tyf, Ey, Hx, Hz, 0, 0, 1, 1, 0, 0, 3, 1);
  if (nx != 1 || ny != 1)  /* Ez: CBx*(Hy - Hy[i-1]) - CBy*(Hx - Hx[j-1]) */
    disp_A_comp(2, 1, nx, 1, ny, 0, nz, nx, ny, nz, P, cE, cD, ID + 2 * NC, (cf*)Tzf, Ez, Hy, Hx, 1, 0, 0, 0, 1, 0, 1, 2);
}

static void disp_B_comp(int i0, int i1, int j0, int j1, int k0, int k1, int nx, int ny, int nz, int P,
                        const cf* cD, const uint32_t* IDc, cf* T, const real* F) {
  const size_t NY = ny + 1, NZ = nz + 1, NC = (size_t)(nx + 1) * NY * NZ;
  int i, j, k, p;
#pragma omp parallel for private(j, k, p) schedule(static)
  for (i = i0; i < i1; i++) for (j = j0; j < j1; j++) for (k = k0; k < k1; k++) {
    const size_t q = IDX(i, j, k);
    const cf* d = cD + 3 * (size_t)P * IDc[q];
    for (p = 0; p < P; p++) T[p * NC + q] = csub(T[p * NC + q], cscale(d[3 * p + 2], F[q]));
  }
}

void oracle_update_dispersive_B(int nx, int ny, int nz, int P, const real* cDf, const uint32_t* ID,
                                real* Txf, real* Tyf, real* Tzf,
                                const real* Ex, const real* Ey, const real* Ez) {
  const size_t NC = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  const cf* cD = (const cf*)cDf;
  if (ny != 1 || nz != 1) disp_B_comp(0, nx, 1, ny, 1, nz, nx, ny, nz, P, cD, ID, (cf*)Txf, Ex);
  if (nx != 1 || nz != 1) disp_B_comp(1, nx, 0, ny, 1, nz, nx, ny, nz, P, cD, ID + NC, (cf*)Tyf, Ey);
  if (nx != 1 || ny != 1) disp_B_comp(1, nx, 1, ny, 0, nz, nx, ny, nz, P, cD, ID + 2 * NC, (cf*)Tzf, Ez);
}

/* magnetic update: fields_updates_ext.pyx:352-412 */
void oracle_update_magnetic(int nx, int ny, int nz, const real* cH, const uint32_t* ID,
                            const real* Ex, const real* Ey, const real* Ez,
                            real* Hx, real* Hy, real* Hz) {
  const size_t NY = ny + 1, NZ = nz + 1, NC = (size_t)(nx + 1) * NY * NZ;
  const uint32_t *IDx = ID + 3 * NC, *IDy = ID + 4 * NC, *IDz = ID + 5 * NC;
  int i, j, k;
  if (nx == 1 || ny == 1 || nz == 1) {
    if (ny == 1 || nz == 1)
      for (i = 1; i < nx; i++) for (j = 0; j < ny; j++) for (k = 0; k < nz; k++) {
        const real* c = cH + 5 * (size_t)IDx[IDX(i, j, k)];
        Hx[IDX(i, j, k)] = c[0] * Hx[IDX(i, j, k)] - c[2] * (Ez[IDX(i, j + 1, k)] - Ez[IDX(i, j, k)]) + c[3] * (Ey[IDX(i, j, k + 1)] - Ey[IDX(i, j, k)]);
      }
    if (nx == 1 || nz == 1)
      for (i = 0; i < nx; i++) for (j = 1; j < ny; j++) for (k = 0; k < nz; k++) {
        const real* c = cH + 5 * (size_t)IDy[IDX(i, j, k)];
        Hy[IDX(i, j, k)] = c[0] * Hy[IDX(i, j, k)] - c[3] * (Ex[IDX(i, j, k + 1)] - Ex[IDX(i, j, k)]) + c[1] * (Ez[IDX(i + 1, j, k)] - Ez[IDX(i, j, k)]);
      }
    if (nx == 1 || ny == 1)
      for (i = 0; i < nx; i++) for (j = 0; j < ny; j++) for (k = 1; k < nz; k++) {
        const real* c = cH + 5 * (size_t)IDz[IDX(i, j, k)];
        Hz[IDX(i, j, k)] = c[0] * Hz[IDX(i, j, k)] - c[1] * (Ey[IDX(i + 1, j, k)] - Ey[IDX(i, j, k)]) + c[2] * (Ex[IDX(i, j + 1, k)] - Ex[IDX(i, j, k)]);
      }
  } else {
#pragma omp parallel for private(j, k) schedule(static)
    for (i = 0; i < nx; i++) for (j = 0; j < ny; j++) for (k = 0; k < nz; k++) {
      const real* a = cH + 5 * (size_t)IDx[IDX(i + 1, j, k)];
      const real* b = cH + 5 * (size_t)IDy[IDX(i, j + 1, k)];
      const real* c = cH + 5 * (size_t)IDz[IDX(i, j, k + 1)];
      Hx[IDX(i + 1, j, k)] = a[0] * Hx[IDX(i + 1, j, k)] - a[2] * (Ez[IDX(i + 1, j + 1, k)] - Ez[IDX(i + 1, j, k)]) + a[3] * (Ey[IDX(i + 1, j, k + 1)] - Ey[IDX(i + 1, j, k)]);
      Hy[IDX(i, j + 1, k)] = b[0] * Hy[IDX(i, j + 1, k)] - b[3] * (Ex[IDX(i, j + 1, k + 1)] - Ex[IDX(i, j + 1, k)]) + b[1] * (Ez[IDX(i + 1, j + 1, k)] - Ez[IDX(i, j + 1, k)]);
      Hz[IDX(i, j, k + 1)] = c[0] * Hz[IDX(i, j, k + 1)] - c[1] * (Ey[IDX(i + 1, j, k + 1)] - Ey[IDX(i, j, k + 1)]) + c[2] * (Ex[IDX(i, j + 1, k + 1)] - Ex[IDX(i, j, k + 1)]);
    }
  }
}

/* ------------------------------------------------------------------------------------
 * PML slab corrections. direction: 0 xminus, 1 yminus, 2 zminus, 3 xplus, 4 yplus, 5 zplus.
 * formulation 0 HORIPML, 1 MRIPML; order 1 or 2. Phi1/Phi2 dims (order, n1, n2, n3) as
 * allocated in gprMax/pml.py:202-219; RA..RF [order][thickness].
 */
typedef struct {
  int xs, xf, ys, yf, zs, zf;
  int p1[3], p2[3];   /* Phi1 / Phi2 dims n1, n2, n3 */
} slab_t;

/* one CFS correction; returns the bracketed term multiplied by the material coefficient */
static inline real pml_step(int form, int order, real dF, real* ph1, real* ph2_order1,
                             const real* RA, const real* RB, const real* RE, const real* RF,
                             int T, int p) {
  /* ph1: Phi[0,...], ph2_order1: Phi[1,...] (second CFS term) */
  if (form == 0 && order == 1) {
    real RA01 = RA[p] - 1, RB0 = RB[p], RE0 = RE[p], RF0 = RF[p];
    real X = RA01 * dF + RB0 * (*ph1);
    *ph1 = RE0 * (*ph1) - RF0 * dF;
    return X;
  } else if (form == 0) {
    real RA0 = RA[p], RB0 = RB[p], RE0 = RE[p], RF0 = RF[p];
    real RA1 = RA[T + p], RB1 = RB[T + p], RE1 = RE[T + p], RF1 = RF[T + p];
    real RA01 = RA[p] * RA[T + p] - 1;
    real X = RA01 * dF + RA1 * RB0 * (*ph1) + RB1 * (*ph2_order1);
    *ph2_order1 = RE1 * (*ph2_order1) - RF1 * (RA0 * dF + RB0 * (*ph1));
    *ph1 = RE0 * (*ph1) - RF0 * dF;
    return X;
  } else if (order == 1) {
    real IRA = 1 / RA[p];
    real IRA1 = IRA - 1;
    real RB0 = RB[p], RE0 = RE[p], RF0 = RF[p];
    real RC0 = IRA * RB0 * RF0;
    real X = IRA1 * dF - IRA * (*ph1);
    *ph1 = RE0 * (*ph1) + RC0 * dF - RC0 * (*ph1);
    return X;
  } else {
    real IRA = 1 / (RA[p] + RA[T + p]);
    real IRA1 = IRA - 1;
    real RB0 = RB[p], RE0 = RE[p], RF0 = RF[p], RC0 = IRA * RF0;
    real RB1 = RB[T + p], RE1 = RE[T + p], RF1 = RF[T + p], RC1 = IRA * RF1;
    real Psi = RB0 * (*ph1) + RB1 * (*ph2_order1);
    real X = IRA1 * dF - IRA * Psi;
    *ph2_order1 = RE1 * (*ph2_order1) + RC1 * (dF - Psi);
    *ph1 = RE0 * (*ph1) + RC0 * (dF - Psi);
    return X;
  }
}

static void pml_generic(int electric, int form, int order, int direction, int xs, int xf, int ys, int yf,
                        int zs, int zf, int gnx, int gny, int gnz, const real* coef, const uint32_t* ID,
                        real* Ex, real* Ey, real* Ez, real* Hx, real* Hy, real* Hz,
                        real* Phi1, real* Phi2, const int* d1, const int* d2,
                        const real* RA, const real* RB, const real* RE, const real* RF, real d) {
  const size_t NY = gny + 1, NZ = gnz + 1, NC = (size_t)(gnx + 1) * NY * NZ;
  const int nxs = xf - xs, nys = yf - ys, nzs = zf - zs;
  const int axis = direction % 3, minus = direction < 3;
  const int T = axis == 0 ? nxs : (axis == 1 ? nys : nzs);
  const size_t o1 = (size_t)d1[0] * d1[1] * d1[2], o2 = (size_t)d2[0] * d2[1] * d2[2];
  /* components: first (Phi1) and second (Phi2) tangential fields, their signs and sources */
  real *F1, *F2;
  const real *S1, *S2;    /* field differenced for F1 / F2 */
  const uint32_t *ID1, *ID2;
  real sg1, sg2;
  int s1i = 0, s1j = 0, s1k = 0;  /* stencil offset along the axis */
  if (electric) {
    if (axis == 0) { F1 = Ey; S1 = Hz; ID1 = ID + NC; sg1 = -1; F2 = Ez; S2 = Hy; ID2 = ID + 2 * NC; sg2 = 1; s1i = 1; }
    else if (axis == 1) { F1 = Ex; S1 = Hz; ID1 = ID; sg1 = 1; F2 = Ez; S2 = Hx; ID2 = ID + 2 * NC; sg2 = -1; s1j = 1; }
    else { F1 = Ex; S1 = Hy; ID1 = ID; sg1 = -1; F2 = Ey; S2 = Hx; ID2 = ID + NC; sg2 = 1; s1k = 1; }
  } else {
    if (axis == 0) { F1 = Hy; S1 = Ez; ID1 = ID + 4 * NC; sg1 = 1; F2 = Hz; S2 = Ey; ID2 = ID + 5 * NC; sg2 = -1; s1i = 1; }
    else if (axis == 1) { F1 = Hx; S1 = Ez; ID1 = ID + 3 * NC; sg1 = -1; F2 = Hz; S2 = Ex; ID2 = ID + 5 * NC; sg2 = 1; s1j = 1; }
    else { F1 = Hx; S1 = Ey; ID1 = ID + 3 * NC; sg1 = 1; F2 = Hy; S2 = Ex; ID2 = ID + 4 * NC; sg2 = -1; s1k = 1; }
  }
  int i, j, k;
#pragma omp parallel for private(j, k) schedule(static)
  for (i = 0; i < nxs; i++) {
    for (j = 0; j < nys; j++) {
      for (k = 0; k < nzs; k++) {
        int ii, jj, kk, p;
        /* node of this slab cell (E: minus ii = xf - i; H: minus ii = xf - (i + 1)) */
        if (axis == 0) { ii = minus ? (electric ? xf - i : xf - (i + 1)) : i + xs; jj = j + ys; kk = k + zs; p = i; }
        else if (axis == 1) { ii = i + xs; jj = minus ? (electric ? yf - j : yf - (j + 1)) : j + ys; kk = k + zs; p = j; }
        else { ii = i + xs; jj = j + ys; kk = minus ? (electric ? zf - k : zf - (k + 1)) : k + zs; p = k; }
        const size_t q = IDX(ii, jj, kk);
        /* E: (F[q] - F[q - 1 along axis]) / d;  H: (F[q + 1 along axis] - F[q]) / d */
        const size_t qa = electric ? IDX(ii - s1i, jj - s1j, kk - s1k) : IDX(ii + s1i, jj + s1j, kk + s1k);
        real dF1 = electric ? (S1[q] - S1[qa]) / d : (S1[qa] - S1[q]) / d;
        real* ph = Phi1 + (((size_t)i * d1[1] + j) * d1[2] + k);
        real X = pml_step(form, order, dF1, ph, ph + o1, RA, RB, RE, RF, T, p);
        const real c1 = coef[5 * (size_t)ID1[q] + 4];
        F1[q] = sg1 > 0 ? F1[q] + c1 * X : F1[q] - c1 * X;
        real dF2 = electric ? (S2[q] - S2[qa]) / d : (S2[qa] - S2[q]) / d;
        ph = Phi2 + (((size_t)i * d2[1] + j) * d2[2] + k);
        X = pml_step(form, order, dF2, ph, ph + o2, RA, RB, RE, RF, T, p);
        const real c2 = coef[5 * (size_t)ID2[q] + 4];
        F2[q] = sg2 > 0 ? F2[q] + c2 * X : F2[q] - c2 * X;
      }
    }
  }
}

void oracle_pml_electric(int form, int order, int direction, int xs, int xf, int ys, int yf, int zs, int zf,
                         int nx, int ny, int nz, const real* cE, const uint32_t* ID,
                         real* Ex, real* Ey, real* Ez, const real* Hx, const real* Hy, const real* Hz,
                         real* Phi1, real* Phi2, const int* d1, const int* d2,
                         const real* RA, const real* RB, const real* RE, const real* RF, real d) {
  pml_generic(1, form, order, direction, xs, xf, ys, yf, zs, zf, nx, ny, nz, cE, ID, Ex, Ey, Ez,
              (real*)Hx, (real*)Hy, (real*)Hz, Phi1, Phi2, d1, d2, RA, RB, RE, RF, d);
}

void oracle_pml_magnetic(int form, int order, int direction, int xs, int xf, int ys, int yf, int zs, int zf,
                         int nx, int ny, int nz, const real* cH, const uint32_t* ID,
                         const real* Ex, const real* Ey, const real* Ez, real* Hx, real* Hy, real* Hz,
                         real* Phi1, real* Phi2, const int* d1, const int* d2,
                         const real* RA, const real* RB, const real* RE, const real* RF, real d) {
  pml_generic(0, form, order, direction, xs, xf, ys, yf, zs, zf, nx, ny, nz, cH, ID, (real*)Ex,
              (real*)Ey, (real*)Ez, Hx, Hy, Hz, Phi1, Phi2, d1, d2, RA, RB, RE, RF, d);
}
