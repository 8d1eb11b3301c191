/*
 * ga_oracle_lin.c - tangent-linear model (TLM) and adjoint of the dry step
 * restated in ga_oracle.c.  Included at the end of ga_oracle.c (it uses that
 * file's static helpers); not compiled on its own.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: the CPU checker of the GPU TLM and
 * adjoint.  The reference has no adjoint; this file's TLM is validated
 * against central finite differences of the oracle's forward step and its
 * adjoint by the dot-product test <L x, y> = <x, L^T y>.  The adjoint is
 * written in scatter form (every forward statement transposed in reverse
 * order), independently of the GPU's gather form.
 *
 * Linearisation conventions:
 *   - upwind signs (signof, fluxes.cpp:295-311) are frozen at the trajectory;
 *   - every face flux of advection has the form a*B + (ab + a)*S
 *     (fluxes.cpp:582-654 with the interpolations of :797-867, :1384-1592):
 *     a the advecting perturbation velocity, ab its basic-state part, B the
 *     basic state of the advected field interpolated with sign(a), S the
 *     advected perturbation interpolated with sign(ab + a).  Its tangent is
 *     dF = (B + S)*da + (ab + a)*dS;
 *   - the pressure solve, projection, boundary conditions and Rayleigh damping
 *     are linear: the TLM applies the forward operators to tangent buffers,
 *     the adjoint applies their transposes;
 *   - the three rotation buffers per field (current, P, M) are part of the
 *     state, as in the forward step (stale lateral rings are carried).
 * Scope: microphysics_option 0, non-periodic lateral boundaries.
 */

struct ora_lin {
    long N;
    double *buf[4][3];
    double *cur[4], *P[4], *M[4];
    double *pi;
};

/* ---- face stencil weights (the face5 / face3 expressions as weights) ---- */
static void weights5(double sg, double *w)
{
    w[0] = one60ths + sg * one60ths;
    w[1] = -two15ths - 5.0 * sg * one60ths;
    w[2] = thirtyseven60ths + 10.0 * sg * one60ths;
    w[3] = thirtyseven60ths - 10.0 * sg * one60ths;
    w[4] = -two15ths + 5.0 * sg * one60ths;
    w[5] = one60ths - sg * one60ths;
}
static void weights3(double sg, double *w)
{
    w[0] = -onetwelfth - sg * onetwelfth;
    w[1] = seventwelfth + 3.0 * sg * onetwelfth;
    w[2] = seventwelfth - 3.0 * sg * onetwelfth;
    w[3] = -onetwelfth + sg * onetwelfth;
}

typedef struct {
    int fa, na;      /* advecting velocity field and its stencil */
    long ia[2];
    double wa[2];
    int fx, ns;      /* advected field and its stencil */
    long is[6];
    double ws[6];
    double ga, gs;   /* dF = ga * da + gs * dS */
} lin_face;

enum { LF_UX, LF_UY, LF_UZ, LF_VX, LF_VY, LF_VZ, LF_TX, LF_TY, LF_TZ };

/* Build the linearised face `fam` at (i,j,k) about S->cur (the trajectory).
 * Returns 0 where the forward flux is identically zero (bottom faces). */
static int lin_face_build(const ora_state *S, int fam, int i, int j, int k, lin_face *L)
{
    const int NZ = S->NZ;
    const int eq = fam / 3, dir = fam % 3;
    const int fx = eq == 0 ? F_U : eq == 1 ? F_V : F_TH;
    const double *X = S->cur[fx], *XB = S->bar[eq == 2 ? 3 : eq];
    if (dir == 2 && k == 0) return 0;
    /* advecting velocity: pairs for momentum, single points for theta */
    int fa = dir; /* u for x faces, v for y faces, w for z faces */
    const double *A = S->cur[fa], *AB = S->bar[fa];
    long a0, a1 = -1;
    if (eq == 2) {
        a0 = dir == 0 ? IX(i + 1, j, k) : dir == 1 ? IX(i, j + 1, k) : IX(i, j, k + 1);
    } else if (eq == 0) {
        if (dir == 0) { a0 = IX(i + 1, j, k); a1 = IX(i, j, k); }
        else if (dir == 1) { a0 = IX(i, j + 1, k); a1 = IX(i - 1, j + 1, k); }
        else { a0 = IX(i, j, k + 1); a1 = IX(i - 1, j, k + 1); }
    } else {
        if (dir == 0) { a0 = IX(i + 1, j, k); a1 = IX(i + 1, j - 1, k); }
        else if (dir == 1) { a0 = IX(i, j + 1, k); a1 = IX(i, j, k); }
        else { a0 = IX(i, j, k + 1); a1 = IX(i, j - 1, k + 1); }
    }
    double a, ab;
    L->fa = fa;
    if (a1 < 0) {
        a = A[a0]; ab = AB[a0];
        L->na = 1; L->ia[0] = a0; L->wa[0] = 1.0;
    } else {
        a = 0.5 * (A[a0] + A[a1]); ab = 0.5 * (AB[a0] + AB[a1]);
        L->na = 2; L->ia[0] = a0; L->ia[1] = a1; L->wa[0] = 0.5; L->wa[1] = 0.5;
    }
    const double sgs = sgn(ab + a), sgb = sgn(a);
    double Sv, Bv;
    L->fx = fx;
    if (dir < 2) {
        long st[6];
        for (int m = 0; m < 6; m++) st[m] = dir == 0 ? IX(i - 2 + m, j, k) : IX(i, j - 2 + m, k);
        Sv = face5(X[st[0]], X[st[1]], X[st[2]], X[st[3]], X[st[4]], X[st[5]], sgs);
        Bv = face5(XB[st[0]], XB[st[1]], XB[st[2]], XB[st[3]], XB[st[4]], XB[st[5]], sgb);
        L->ns = 6;
        weights5(sgs, L->ws);
        for (int m = 0; m < 6; m++) L->is[m] = st[m];
    } else if (k == 1 || k == NZ - 2) {
        long p0 = IX(i, j, k), p1 = IX(i, j, k + 1);
        Sv = 0.5 * (X[p1] + X[p0]);
        Bv = 0.5 * (XB[p1] + XB[p0]);
        L->ns = 2; L->is[0] = p0; L->is[1] = p1; L->ws[0] = 0.5; L->ws[1] = 0.5;
    } else {
        long st[4];
        for (int m = 0; m < 4; m++) st[m] = IX(i, j, k - 1 + m);
        Sv = face3(X[st[0]], X[st[1]], X[st[2]], X[st[3]], sgs);
        Bv = face3(XB[st[0]], XB[st[1]], XB[st[2]], XB[st[3]], sgb);
        L->ns = 4;
        weights3(sgs, L->ws);
        for (int m = 0; m < 4; m++) L->is[m] = st[m];
    }
    L->ga = Bv + Sv;
    L->gs = ab + a;
    return 1;
}

static double lin_face_tl(const ora_state *S, const ora_lin *T, int fam, int i, int j, int k)
{
    lin_face L;
    if (!lin_face_build(S, fam, i, j, k, &L)) return 0.0;
    const double *dA = T->cur[L.fa], *dX = T->cur[L.fx];
    double da = 0, ds = 0;
    for (int m = 0; m < L.na; m++) da += L.wa[m] * dA[L.ia[m]];
    for (int m = 0; m < L.ns; m++) ds += L.ws[m] * dX[L.is[m]];
    return L.ga * da + L.gs * ds;
}

static void lin_face_ad(const ora_state *S, ora_lin *A, int fam, int i, int j, int k, double fbar)
{
    lin_face L;
    if (fbar == 0.0 || !lin_face_build(S, fam, i, j, k, &L)) return;
    double *aA = A->cur[L.fa], *aX = A->cur[L.fx];
    const double abar = L.ga * fbar, sbar = L.gs * fbar;
    for (int m = 0; m < L.na; m++) aA[L.ia[m]] += L.wa[m] * abar;
    for (int m = 0; m < L.ns; m++) aX[L.is[m]] += L.ws[m] * sbar;
}

/* tangent of the tendency of equation eq (0 u, 1 v, 2 theta) at a cell */
static double tl_tend(const ora_state *S, const ora_lin *T, int eq, int i, int j, int k)
{
    const double *rhow = S->rhow, *odr = S->one_d_rhou;
    const double DTZ = S->dtz * S->mu[k];
    const int f0 = 3 * eq;
    double t = -S->dtx * (lin_face_tl(S, T, f0, i, j, k) - lin_face_tl(S, T, f0, i - 1, j, k)) -
               S->dty * (lin_face_tl(S, T, f0 + 1, i, j, k) - lin_face_tl(S, T, f0 + 1, i, j - 1, k)) -
               DTZ * (rhow[k + 1] * lin_face_tl(S, T, f0 + 2, i, j, k) -
                      rhow[k] * lin_face_tl(S, T, f0 + 2, i, j, k - 1)) * odr[k];
    if (eq == 0) {
        const double *dV = T->cur[F_V];
        t += S->dt * S->f[j] * 0.25 *
             (dV[IX(i, j, k)] + dV[IX(i, j + 1, k)] + dV[IX(i - 1, j, k)] + dV[IX(i - 1, j + 1, k)]);
    } else if (eq == 1) {
        const double *dU = T->cur[F_U];
        t -= S->dt * S->f[j] * 0.25 *
             (dU[IX(i, j, k)] + dU[IX(i + 1, j, k)] + dU[IX(i, j - 1, k)] + dU[IX(i + 1, j - 1, k)]);
    } else {
        const double *dW = T->cur[F_W], *tb = S->tb;
        t -= DTZ * 0.5 *
             (rhow[k + 1] * dW[IX(i, j, k + 1)] * (tb[k + 1] - tb[k]) +
              rhow[k] * dW[IX(i, j, k)] * (tb[k] - tb[k - 1])) * odr[k];
    }
    return t;
}

/* transpose of tl_tend: scatter tbar (the adjoint of the tendency) */
static void ad_tend(const ora_state *S, ora_lin *A, int eq, int i, int j, int k, double tbar)
{
    if (tbar == 0.0) return;
    const double *rhow = S->rhow, *odr = S->one_d_rhou;
    const double DTZ = S->dtz * S->mu[k];
    const int f0 = 3 * eq;
    lin_face_ad(S, A, f0, i, j, k, -S->dtx * tbar);
    lin_face_ad(S, A, f0, i - 1, j, k, S->dtx * tbar);
    lin_face_ad(S, A, f0 + 1, i, j, k, -S->dty * tbar);
    lin_face_ad(S, A, f0 + 1, i, j - 1, k, S->dty * tbar);
    lin_face_ad(S, A, f0 + 2, i, j, k, -DTZ * rhow[k + 1] * odr[k] * tbar);
    lin_face_ad(S, A, f0 + 2, i, j, k - 1, DTZ * rhow[k] * odr[k] * tbar);
    if (eq == 0) {
        double *aV = A->cur[F_V];
        const double c = S->dt * S->f[j] * 0.25 * tbar;
        aV[IX(i, j, k)] += c; aV[IX(i, j + 1, k)] += c;
        aV[IX(i - 1, j, k)] += c; aV[IX(i - 1, j + 1, k)] += c;
    } else if (eq == 1) {
        double *aU = A->cur[F_U];
        const double c = S->dt * S->f[j] * 0.25 * tbar;
        aU[IX(i, j, k)] -= c; aU[IX(i + 1, j, k)] -= c;
        aU[IX(i, j - 1, k)] -= c; aU[IX(i + 1, j - 1, k)] -= c;
    } else {
        double *aW = A->cur[F_W];
        const double *tb = S->tb;
        aW[IX(i, j, k + 1)] -= DTZ * 0.5 * rhow[k + 1] * (tb[k + 1] - tb[k]) * odr[k] * tbar;
        aW[IX(i, j, k)] -= DTZ * 0.5 * rhow[k] * (tb[k] - tb[k - 1]) * odr[k] * tbar;
    }
}

/* ---- advection operators ---- */
static void tl_advect_uvw(const ora_state *S, ora_lin *T, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 1; k < NZ - 1; k++) {
                long c = IX(i, j, k);
                T->P[F_U][c] = T->M[F_U][c] + step * tl_tend(S, T, 0, i, j, k);
                T->P[F_V][c] = T->M[F_V][c] + step * tl_tend(S, T, 1, i, j, k);
            }
    const double *dTH = T->cur[F_TH], *tbv = S->tbv;
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 2; k < NZ - 1; k++) {
                long c = IX(i, j, k);
                double b0 = dTH[c] / tbv[k], b1 = dTH[c - 1] / tbv[k - 1];
                T->P[F_W][c] = T->M[F_W][c] + step * S->dt * grav * 0.5 * (b0 + b1);
            }
}

static void ad_advect_uvw(const ora_state *S, ora_lin *A, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    double *aTH = A->cur[F_TH];
    const double *tbv = S->tbv;
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 2; k < NZ - 1; k++) {
                long c = IX(i, j, k);
                double pb = A->P[F_W][c];
                A->M[F_W][c] += pb;
                double g = step * S->dt * grav * 0.5 * pb;
                aTH[c] += g / tbv[k];
                aTH[c - 1] += g / tbv[k - 1];
                A->P[F_W][c] = 0;
            }
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 1; k < NZ - 1; k++) {
                long c = IX(i, j, k);
                double pu = A->P[F_U][c], pv = A->P[F_V][c];
                A->M[F_U][c] += pu;
                A->M[F_V][c] += pv;
                A->P[F_U][c] = 0;
                A->P[F_V][c] = 0;
                ad_tend(S, A, 0, i, j, k, step * pu);
                ad_tend(S, A, 1, i, j, k, step * pv);
            }
}

static void tl_advect_theta(const ora_state *S, ora_lin *T, double step)
{
    for (int i = 3; i < S->NX - 3; i++)
        for (int j = 3; j < S->NY - 3; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                long c = IX(i, j, k);
                T->P[F_TH][c] = T->M[F_TH][c] + step * tl_tend(S, T, 2, i, j, k);
            }
}

static void ad_advect_theta(const ora_state *S, ora_lin *A, double step)
{
    for (int i = 3; i < S->NX - 3; i++)
        for (int j = 3; j < S->NY - 3; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                long c = IX(i, j, k);
                double pt = A->P[F_TH][c];
                A->M[F_TH][c] += pt;
                A->P[F_TH][c] = 0;
                ad_tend(S, A, 2, i, j, k, step * pt);
            }
}

/* ---- transposes of the linear operators ---- */
static void mirror_ad(const ora_state *S, double *s) /* transpose of mirror() */
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    for (int k = 1; k < NZ - 1; k++) {
        for (int i = 0; i < NX; i++) {
            s[IX(i, 1, k)] += s[IX(i, 0, k)]; s[IX(i, 0, k)] = 0;
            s[IX(i, NY - 2, k)] += s[IX(i, NY - 1, k)]; s[IX(i, NY - 1, k)] = 0;
        }
        for (int j = 0; j < NY; j++) {
            s[IX(1, j, k)] += s[IX(0, j, k)]; s[IX(0, j, k)] = 0;
            s[IX(NX - 2, j, k)] += s[IX(NX - 1, j, k)]; s[IX(NX - 1, j, k)] = 0;
        }
    }
}

/* Transpose of poisson(): pi -> (P_u, P_v, P_w).  The forward map is
 * Re(G T F d) / (ni nj) with F, G the forward and inverse 2-D DFTs and T the
 * per-wavenumber tridiagonal solve; its transpose is Re(G T^T F y) / (ni nj). */
static void poisson_ad(ora_state *S, ora_lin *A, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    const int ni = S->ni, nj = S->nj, nk = S->nk;
    double *PI = A->pi;
    memset(S->spec, 0, sizeof(double) * 2 * (size_t)ni * nj * nk);
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < nj; j++) {
            for (int k = 1; k < nk - 1; k++) SP(i, j, k)[0] = PI[IX(i, j, k)];
            SP(i, j, 1)[0] += PI[IX(i, j, 0)];
            SP(i, j, NZ - 2)[0] += PI[IX(i, j, NZ - 1)];
        }
    memset(PI, 0, sizeof(double) * S->N);
    for (int k = 1; k < nk - 1; k++) {
        ora_fft_2d(&S->fi, &S->fj, -1, SP(0, 0, k), S->specw);
        memcpy(SP(0, 0, k), S->specw, sizeof(double) * 2 * (size_t)ni * nj);
    }
    /* transposed Thomas: h = U^-T y, gauge, e = L^-T h */
    double *F = (double *)malloc(sizeof(double) * nk), *Z = (double *)malloc(sizeof(double) * nk);
    const double dx2 = S->dx * S->dx;
    const int K = NZ - 2;
    for (int p = 0; p < ni; p++)
        for (int q = 0; q < nj; q++) {
            double h = S->hcoef[(long)p * nj + q];
            Z[1] = 1.0 / (S->rhou[1] * 2.0 * h / dx2 - S->vcoef[1]);
            F[1] = S->ccoef[1] * Z[1];
            for (int k = 2; k < nk - 1; k++) {
                double b = S->rhou[k] * 2.0 * h / dx2 - S->vcoef[k];
                Z[k] = 1.0 / (b - S->acoef[k] * F[k - 1]);
                F[k] = S->ccoef[k] * Z[k];
            }
            for (int c = 0; c < 2; c++) {
                for (int k = 2; k <= K; k++) SP(p, q, k)[c] -= F[k - 1] * SP(p, q, k - 1)[c];
                /* mean mode: the gauge removes row K, so z_K (infinite there)
                 * never enters the map and its adjoint entry is zero */
                if (p == 0 && q == 0) SP(p, q, K)[c] = 0;
                else SP(p, q, K)[c] *= Z[K];
                for (int k = K - 1; k >= 1; k--)
                    SP(p, q, k)[c] = Z[k] * (SP(p, q, k)[c] - S->acoef[k + 1] * SP(p, q, k + 1)[c]);
            }
        }
    free(F);
    free(Z);
    const double size2d = (double)(ni * nj);
    for (int k = 1; k < nk - 1; k++) {
        ora_fft_2d(&S->fi, &S->fj, +1, SP(0, 0, k), S->specw);
        for (long x = 0; x < (long)ni * nj; x++) {
            SP(0, 0, k)[2 * x] = S->specw[2 * x] / size2d;
            SP(0, 0, k)[2 * x + 1] = 0;
        }
    }
    /* transposed lateral copies of the divergence (j copies were applied last) */
    for (int k = 1; k < NZ - 1; k++) {
        for (int i = 0; i < ni; i++) {
            SP(i, 1, k)[0] += SP(i, 0, k)[0]; SP(i, 0, k)[0] = 0;
            SP(i, NY - 2, k)[0] += SP(i, NY - 1, k)[0]; SP(i, NY - 1, k)[0] = 0;
        }
        for (int j = 0; j < NY; j++) {
            SP(1, j, k)[0] += SP(0, j, k)[0]; SP(0, j, k)[0] = 0;
            SP(NX - 2, j, k)[0] += SP(NX - 1, j, k)[0]; SP(NX - 1, j, k)[0] = 0;
        }
    }
    double *aU = A->P[F_U], *aV = A->P[F_V], *aW = A->P[F_W];
    const double *rhou = S->rhou, *rhow = S->rhow;
    for (int i = 1; i < NX - 1; i++)
        for (int j = 1; j < NY - 1; j++)
            for (int k = 1; k < NZ - 1; k++) {
                double d = SP(i, j, k)[0] / (step * S->dt);
                double cu = rhou[k] * S->one_d_dx * d, cv = rhou[k] * S->one_d_dy * d;
                double cw = S->one_d_dz * S->mu[k] * d;
                aU[IX(i + 1, j, k)] += cu; aU[IX(i, j, k)] -= cu;
                aV[IX(i, j + 1, k)] += cv; aV[IX(i, j, k)] -= cv;
                aW[IX(i, j, k + 1)] += rhow[k + 1] * cw; aW[IX(i, j, k)] -= rhow[k] * cw;
            }
}

static void ad_solve_pressure(ora_state *S, ora_lin *A, double step)
{
    mirror_ad(S, A->pi);
    poisson_ad(S, A, step);
    mirror_ad(S, A->P[F_W]);
    mirror_ad(S, A->P[F_V]);
    mirror_ad(S, A->P[F_U]);
}

static void ad_project(const ora_state *S, ora_lin *A, double step)
{
    const double *UP = A->P[F_U], *VP = A->P[F_V], *WP = A->P[F_W];
    double *PI = A->pi;
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++) {
            for (int k = 1; k < S->NZ - 1; k++) {
                double cu = step * S->dtx * UP[IX(i, j, k)], cv = step * S->dty * VP[IX(i, j, k)];
                PI[IX(i, j, k)] -= cu; PI[IX(i - 1, j, k)] += cu;
                PI[IX(i, j, k)] -= cv; PI[IX(i, j - 1, k)] += cv;
                if (k >= 2) {
                    double cw = step * (S->dtz * S->mw[k]) * WP[IX(i, j, k)];
                    PI[IX(i, j, k)] -= cw; PI[IX(i, j, k - 1)] += cw;
                }
            }
        }
}

static void upper_lower_ad(const ora_state *S, double *v)
{
    for (int i = 1; i < S->NX; i++)
        for (int j = 1; j < S->NY; j++) {
            v[IX(i, j, S->NZ - 2)] += v[IX(i, j, S->NZ - 1)]; v[IX(i, j, S->NZ - 1)] = 0;
            v[IX(i, j, 1)] += v[IX(i, j, 0)]; v[IX(i, j, 0)] = 0;
        }
}

static void ad_bc(ora_state *S, ora_lin *A)
{
    upper_lower_zero(S, A->P[F_W]);
    sponge(S, A->P[F_W], 0);
    upper_lower_ad(S, A->P[F_TH]);
    upper_lower_ad(S, A->P[F_V]);
    upper_lower_ad(S, A->P[F_U]);
    sponge(S, A->P[F_TH], 0);
    sponge(S, A->P[F_V], 0);
    sponge(S, A->P[F_U], 0);
}

/* run a linear forward operator on the buffers of L */
static void lin_exchange(ora_state *S, ora_lin *L)
{
    for (int f = 0; f < 4; f++) {
        double *t;
        t = S->cur[f]; S->cur[f] = L->cur[f]; L->cur[f] = t;
        t = S->P[f]; S->P[f] = L->P[f]; L->P[f] = t;
        t = S->M[f]; S->M[f] = L->M[f]; L->M[f] = t;
    }
    double *t = S->pi; S->pi = L->pi; L->pi = t;
}

static void lin_swap_inner(ora_lin *L)
{
    for (int f = 0; f < 4; f++) { double *t = L->cur[f]; L->cur[f] = L->P[f]; L->P[f] = t; }
}

static const double rk3_steps[3] = {1. / 3., 0.5, 1.0};

/* One forward step of S with the stage-start current fields (u, v, w, theta)
 * copied into rec[(s*4 + f)*N] (rec may be NULL), and the matching tangent
 * step of T (T may be NULL). */
static void rk3_step_lin(ora_state *S, ora_lin *T, double *rec)
{
    for (int s = 0; s < 3; s++) {
        const double st = rk3_steps[s];
        if (rec)
            for (int f = 0; f < 4; f++) memcpy(rec + (size_t)(s * 4 + f) * S->N, S->cur[f], sizeof(double) * S->N);
        if (T) {
            tl_advect_uvw(S, T, st);
            tl_advect_theta(S, T, st);
            lin_exchange(S, T);
            op_solve_pressure(S, st);
            op_project(S, st);
            op_bc(S);
            lin_exchange(S, T);
            if (s < 2) lin_swap_inner(T);
        }
        integrate_non_hydro(S, st);
        op_advect_theta(S, st);
        op_bc(S);
        if (s < 2) advance_inner(S);
    }
    op_bc(S);
    op_rayleigh(S);
    advance_outer(S);
    S->mtime += S->dt;
    S->bigcounter++;
    if (T) {
        lin_exchange(S, T);
        op_bc(S);
        op_rayleigh(S);
        lin_exchange(S, T);
        for (int f = 0; f < 4; f++) memcpy(T->M[f], T->P[f], sizeof(double) * T->N);
        lin_swap_inner(T);
    }
}

/* adjoint of one step about the trajectory recorded in rec */
static void adj_step(ora_state *S, ora_lin *A, const double *rec)
{
    const long N = S->N;
    lin_swap_inner(A);
    for (int f = 0; f < 4; f++)
        for (long x = 0; x < N; x++) { A->P[f][x] += A->M[f][x]; A->M[f][x] = 0; }
    lin_exchange(S, A);
    op_rayleigh(S);
    lin_exchange(S, A);
    ad_bc(S, A);
    double *saved[4];
    for (int f = 0; f < 4; f++) saved[f] = S->cur[f];
    for (int s = 2; s >= 0; s--) {
        const double st = rk3_steps[s];
        if (s < 2) lin_swap_inner(A);
        for (int f = 0; f < 4; f++) S->cur[f] = (double *)rec + (size_t)(s * 4 + f) * N;
        ad_bc(S, A);
        ad_advect_theta(S, A, st);
        ad_project(S, A, st);
        ad_solve_pressure(S, A, st);
        ad_advect_uvw(S, A, st);
    }
    for (int f = 0; f < 4; f++) S->cur[f] = saved[f];
}

/* ---- API ---- */
static int lin_supported(const ora_state *S)
{
    return S->c.microphysics_option == 0 && !S->c.periodic_ew_boundaries;
}

ora_lin *ora_lin_create(ora_state *S)
{
    if (!S || !lin_supported(S)) return NULL;
    ora_lin *L = (ora_lin *)calloc(1, sizeof(ora_lin));
    L->N = S->N;
    for (int f = 0; f < 4; f++) {
        for (int s = 0; s < 3; s++) L->buf[f][s] = (double *)calloc((size_t)S->N, sizeof(double));
        L->cur[f] = L->buf[f][0];
        L->P[f] = L->buf[f][1];
        L->M[f] = L->buf[f][2];
    }
    L->pi = (double *)calloc((size_t)S->N, sizeof(double));
    return L;
}

void ora_lin_destroy(ora_lin *L)
{
    if (!L) return;
    for (int f = 0; f < 4; f++)
        for (int s = 0; s < 3; s++) free(L->buf[f][s]);
    free(L->pi);
    free(L);
}

static double *lin_ptr(ora_lin *L, int field, int slot)
{
    if (field == GA_PI) return L->pi;
    if (field < 0 || field >= 4) return NULL;
    if (slot == GA_SLOT_CUR) return L->cur[field];
    if (slot == GA_SLOT_P) return L->P[field];
    if (slot == GA_SLOT_M) return L->M[field];
    return NULL;
}

int ora_lin_set(ora_lin *L, int field, int slot, const double *src, long n)
{
    double *d = lin_ptr(L, field, slot);
    if (!d || n != L->N) return GA_ERR_ARG;
    memcpy(d, src, sizeof(double) * n);
    return GA_OK;
}

int ora_lin_get(ora_lin *L, int field, int slot, double *dst, long n)
{
    double *d = lin_ptr(L, field, slot);
    if (!d || n != L->N) return GA_ERR_ARG;
    memcpy(dst, d, sizeof(double) * n);
    return GA_OK;
}

int ora_tlm_step(ora_state *S, ora_lin *T, int nsteps)
{
    if (!S || !T || !lin_supported(S)) return GA_ERR_UNSUPPORTED;
    for (int n = 0; n < nsteps; n++) rk3_step_lin(S, T, NULL);
    return GA_OK;
}

int ora_adj_run(ora_state *S, ora_lin *A, int nsteps)
{
    if (!S || !A || !lin_supported(S)) return GA_ERR_UNSUPPORTED;
    double *rec = (double *)malloc(sizeof(double) * (size_t)nsteps * 12 * S->N);
    if (!rec) return GA_ERR_NOMEM;
    for (int n = 0; n < nsteps; n++) rk3_step_lin(S, NULL, rec + (size_t)n * 12 * S->N);
    for (int n = nsteps - 1; n >= 0; n--) adj_step(S, A, rec + (size_t)n * 12 * S->N);
    free(rec);
    return GA_OK;
}
