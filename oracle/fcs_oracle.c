/*
 * fcs_oracle.c -- CPU restatement of the reference per-cell stiff chemistry
 * path.  TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference leg of bench.py as the checker; never by the
 * product library.
 *
 * Reference files restated here (paths inside the reference project):
 *   mechanism ordering    src/Reaction/OptReaction.C:348-1339
 *   thermo                src/Reaction/ThermoFunctionI.H:1-31, 33-371, 539-636, 799-881
 *   rates (dNdtByV)       src/Reaction/ReactionRate.C:732-1503, ReactionFunctionI.H:1-721,
 *                         ChemicalEquilibriumFunctionI.H:14-25
 *   Jacobian              src/Reaction/Jacobian.C:5-1004, JacobianFunctionI.H (JF11..JF33, JFG)
 *   dC/dY conversion      src/Reaction/Jacobian.C:2814-2858 (exact), 3709-3741 (T column),
 *                         3743-3793 (T row), 4541-4568 (fast)
 *   model closure         src/ChemistryModel/FastChemistryModel.C:194-273, 340-417, 489-572
 *   LU                    src/LUsolver/LUsolver.C:106-246, 503-660, 3058-3143, 4113-4152
 *   Rodas34               src/ODE/OptRodas34/OptRodas34.C:57-882, OptRodas34.H:105-149
 *   Rosenbrock34          src/ODE/OptRosenbrock34/OptRosenbrock34.C:61-678, .H:117-158
 *   Seulex                src/ODE/OptSeulex/OptSeulex.C:34-734, .H:130-175
 *   cell loop             src/ChemistryModel/FastChemistryModel_transientSolve.H:30-104
 */
#include "fcs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define RU 8314.470066505449722171761095523834228515625
#define PSTD 100000.0
#define KC_CLAMP 1.4901171103413047e-8
#define KC_CLAMP_G 1.49011611938476E-08
#define PIV_EPS 2.2204460492503131e-16
#define SMALL 1.0e-15
#define VGREAT 1.0e300
#define IS_FALLOFF(k) ((k) >= FCS_RXN_LINDEMANN_FALLOFF && (k) <= FCS_RXN_SRI_FALLOFF)
#define IS_NONEQ(k) ((k) == FCS_RXN_NONEQ || (k) == FCS_RXN_NONEQ_THIRD_BODY)
/* kinds that take a third-body row: M = E C */
#define HAS_TB(k) ((k) == FCS_RXN_THIRD_BODY || (k) == FCS_RXN_NONEQ_THIRD_BODY || IS_FALLOFF(k))

struct orc_mech {
    int ns, n, nr;
    double *W, *invW, *Tcommon, *coef; /* coef [ns][2][7]: [0] low, [1] high */
    double TlowMin, ThighMax, TcommonMin, TcommonMax;
    int nTI, nArr, nTB, nFO, nPlog;
    /* per reaction, reference order */
    int *kind, *rev, *fileIdx, *lOff, *lSp, *rOff, *rSp, *tbRow, *plogIdx, *dnu;
    double *A, *beta, *Ta;
    double *A2, *beta2, *Ta2;    /* per reaction: kInf of fall-off, reverse rate of non-equilibrium */
    double *fo;                  /* [nr][5] Troe (alpha, Ts, Tss, Tsss) / SRI (a, b, c, d, e) */
    double *eff;                 /* [nTB][ns]: non-equilibrium third-body, third-body, then fall-off rows */
    int *pOff;                   /* [nPlog+1] */
    double *pP, *pLogP, *pLogA, *pBeta, *pTa;
    int maxSp;
};

int32_t orc_mech_n_species(const orc_mech* m) { return m->ns; }

int32_t orc_mech_order(const orc_mech* m, int32_t* out)
{
    for (int i = 0; i < m->nr; i++) out[i] = m->fileIdx[i];
    return m->nr;
}

void orc_mech_destroy(orc_mech* m)
{
    if (!m) return;
    free(m->W); free(m->invW); free(m->Tcommon); free(m->coef);
    free(m->kind); free(m->rev); free(m->fileIdx); free(m->lOff); free(m->lSp);
    free(m->rOff); free(m->rSp); free(m->tbRow); free(m->plogIdx); free(m->dnu);
    free(m->A); free(m->beta); free(m->Ta); free(m->eff); free(m->pOff);
    free(m->A2); free(m->beta2); free(m->Ta2); free(m->fo);
    free(m->pP); free(m->pLogP); free(m->pLogA); free(m->pBeta); free(m->pTa);
    free(m);
}

/* Type-block order of OptReaction::readInfo (OptReaction.C:448-1175):
 * temperature-independent Arrhenius, other Arrhenius, non-equilibrium,
 * non-equilibrium third-body (OptReaction.C:610-700), third-body, fall-off
 * (Lindemann, then Troe, then SRI: OptReaction.C:746-917), (chemically
 * activated), PLOG; file order inside each block.  Third-body rows follow the
 * same order (Itbr[0..3]); rev is 2 for non-equilibrium reactions
 * (isIrreversible = 2, OptReaction.C:619, 654), whose reverse rate is their
 * own Arrhenius.  The reference builds the reverse third-body row of a
 * non-equilibrium reaction from the forward coefficients (OptReaction.C:678),
 * so one row serves both directions. */
orc_mech* orc_mech_create(const fcs_mechanism_desc* d, int32_t* status)
{
    *status = FCS_OK;
    const int ns = d->n_species, nr = d->n_reactions;
    for (int r = 0; r < nr; r++) {
        int t = d->type[r];
        if (t < FCS_RXN_ARRHENIUS || t > FCS_RXN_NONEQ_THIRD_BODY) {
            *status = FCS_ERR_UNSUPPORTED;
            return NULL;
        }
    }
    orc_mech* m = (orc_mech*)calloc(1, sizeof(orc_mech));
    m->ns = ns; m->n = ns + 1; m->nr = nr;
    m->W = (double*)malloc(sizeof(double) * ns);
    m->invW = (double*)malloc(sizeof(double) * ns);
    m->Tcommon = (double*)malloc(sizeof(double) * ns);
    m->coef = (double*)malloc(sizeof(double) * ns * 14);
    m->TlowMin = 1e10; m->ThighMax = 1; m->TcommonMin = 1e10; m->TcommonMax = 0;
    for (int i = 0; i < ns; i++) {
        m->W[i] = d->W[i];
        m->invW[i] = 1.0 / d->W[i];
        m->Tcommon[i] = d->T_common[i];
        memcpy(&m->coef[i * 14], &d->low_coeffs[i * 7], 7 * sizeof(double));
        memcpy(&m->coef[i * 14 + 7], &d->high_coeffs[i * 7], 7 * sizeof(double));
        if (m->TlowMin > d->T_low[i]) m->TlowMin = d->T_low[i];
        if (m->ThighMax < d->T_high[i]) m->ThighMax = d->T_high[i];
        if (d->T_common[i] > m->TcommonMax) m->TcommonMax = d->T_common[i];
        if (d->T_common[i] < m->TcommonMin) m->TcommonMin = d->T_common[i];
    }
    int* order = (int*)malloc(sizeof(int) * (nr > 0 ? nr : 1));
    int k = 0;
    for (int pass = 0; pass < 9; pass++) {
        for (int r = 0; r < nr; r++) {
            int t = d->type[r];
            double beta = d->arrhenius[3 * r + 1], Ta = d->arrhenius[3 * r + 2];
            int tind = (beta == 0 && Ta == 0);
            if ((pass == 0 && t == FCS_RXN_ARRHENIUS && tind) ||
                (pass == 1 && t == FCS_RXN_ARRHENIUS && !tind) ||
                (pass == 2 && t == FCS_RXN_NONEQ) ||
                (pass == 3 && t == FCS_RXN_NONEQ_THIRD_BODY) ||
                (pass == 4 && t == FCS_RXN_THIRD_BODY) ||
                (pass == 5 && t == FCS_RXN_LINDEMANN_FALLOFF) ||
                (pass == 6 && t == FCS_RXN_TROE_FALLOFF) ||
                (pass == 7 && t == FCS_RXN_SRI_FALLOFF) ||
                (pass == 8 && t == FCS_RXN_PLOG))
                order[k++] = r;
        }
    }
#define ALLOC_I(x, n) x = (int*)calloc((n) > 0 ? (n) : 1, sizeof(int))
#define ALLOC_D(x, n) x = (double*)calloc((n) > 0 ? (n) : 1, sizeof(double))
    ALLOC_I(m->kind, nr); ALLOC_I(m->rev, nr); ALLOC_I(m->fileIdx, nr);
    ALLOC_I(m->lOff, nr + 1); ALLOC_I(m->rOff, nr + 1); ALLOC_I(m->tbRow, nr);
    ALLOC_I(m->plogIdx, nr); ALLOC_I(m->dnu, nr);
    ALLOC_D(m->A, nr); ALLOC_D(m->beta, nr); ALLOC_D(m->Ta, nr);
    ALLOC_D(m->A2, nr); ALLOC_D(m->beta2, nr); ALLOC_D(m->Ta2, nr); ALLOC_D(m->fo, (size_t)nr * 5);
    int nl_tot = d->lhs_offset[nr], nr_tot = d->rhs_offset[nr];
    ALLOC_I(m->lSp, nl_tot); ALLOC_I(m->rSp, nr_tot);
    int nTB = 0, nPlog = 0, plogRows = 0;
    for (int r = 0; r < nr; r++) {
        if (HAS_TB(d->type[r])) nTB++;
        if (IS_FALLOFF(d->type[r])) m->nFO++;
        if (d->type[r] == FCS_RXN_PLOG) { nPlog++; plogRows += d->plog_offset[r + 1] - d->plog_offset[r]; }
    }
    m->nTB = nTB; m->nPlog = nPlog;
    ALLOC_D(m->eff, nTB * ns);
    ALLOC_I(m->pOff, nPlog + 1);
    ALLOC_D(m->pP, plogRows); ALLOC_D(m->pLogP, plogRows); ALLOC_D(m->pLogA, plogRows);
    ALLOC_D(m->pBeta, plogRows); ALLOC_D(m->pTa, plogRows);
    int lo = 0, ro = 0, tb = 0, pl = 0, prow = 0;
    m->maxSp = 0;
    for (int i = 0; i < nr; i++) {
        int r = order[i];
        m->fileIdx[i] = r;
        m->kind[i] = d->type[r];
        m->rev[i] = IS_NONEQ(d->type[r]) ? 2 : d->reversible[r] ? 1 : 0;
        m->A[i] = d->arrhenius[3 * r + 0];
        m->beta[i] = d->arrhenius[3 * r + 1];
        m->Ta[i] = d->arrhenius[3 * r + 2];
        m->lOff[i] = lo;
        for (int j = d->lhs_offset[r]; j < d->lhs_offset[r + 1]; j++) m->lSp[lo++] = d->lhs_species[j];
        m->rOff[i] = ro;
        for (int j = d->rhs_offset[r]; j < d->rhs_offset[r + 1]; j++) m->rSp[ro++] = d->rhs_species[j];
        int nlr = d->lhs_offset[r + 1] - d->lhs_offset[r];
        int nrr = d->rhs_offset[r + 1] - d->rhs_offset[r];
        if (nlr > m->maxSp) m->maxSp = nlr;
        if (nrr > m->maxSp) m->maxSp = nrr;
        m->dnu[i] = nrr - nlr;
        m->tbRow[i] = -1;
        m->plogIdx[i] = -1;
        if (HAS_TB(m->kind[i])) {
            for (int s = 0; s < ns; s++) m->eff[tb * ns + s] = d->efficiencies[(size_t)r * ns + s];
            m->tbRow[i] = tb++;
        }
        if (IS_FALLOFF(m->kind[i]) || IS_NONEQ(m->kind[i])) {
            m->A2[i] = d->arrhenius2[3 * r + 0];
            m->beta2[i] = d->arrhenius2[3 * r + 1];
            m->Ta2[i] = d->arrhenius2[3 * r + 2];
        }
        if (IS_FALLOFF(m->kind[i]))
            for (int q = 0; q < 5; q++) m->fo[(size_t)i * 5 + q] = d->falloff_params[(size_t)r * 5 + q];
        if (m->kind[i] == FCS_RXN_PLOG) {
            m->plogIdx[i] = pl;
            m->pOff[pl] = prow;
            for (int q = d->plog_offset[r]; q < d->plog_offset[r + 1]; q++) {
                const double* row = &d->plog_table[4 * q];
                m->pP[prow] = row[0];
                m->pLogP[prow] = log(row[0]);
                m->pLogA[prow] = log(row[1]);
                m->pBeta[prow] = row[2];
                m->pTa[prow] = row[3];
                prow++;
            }
            pl++;
        }
        if (m->kind[i] == FCS_RXN_ARRHENIUS) {
            m->nArr++;
            if (m->beta[i] == 0 && m->Ta[i] == 0) m->nTI++;
        }
    }
    m->pOff[pl] = prow;
    m->lOff[nr] = lo; m->rOff[nr] = ro;
    free(order);
    return m;
}

/* ------------------------------------------------------------------------ */
/* per-thread workspace                                                      */

typedef struct {
    const orc_mech* m;
    int n;
    double *C, *B, *dBdT, *Cp, *Ha, *dCpdT, *rhoMvj, *WiByrhoM;
    double *Kf, *dKfdT, *M, *Kplog, *dKplog;
    double *Kinf, *dKinfdT;      /* second Arrhenius: kInf (fall-off), reverse rate (non-equilibrium) */
    double *Jc, *Jy, *a;       /* N*N each */
    double *vec[16];           /* N each */
    int *piv;
    double *invD;
    double *table;             /* Seulex: 12*N */
    double rhoM;               /* last thermo rhoM (kg/m3) */
    double invT;
    int64_t cnt[ORC_NCOUNTERS];
} ws_t;

static ws_t* ws_create(const orc_mech* m)
{
    ws_t* w = (ws_t*)calloc(1, sizeof(ws_t));
    int n = m->n, ns = m->ns, nr = m->nr;
    w->m = m; w->n = n;
    w->C = (double*)calloc(ns, sizeof(double));
    w->B = (double*)calloc(ns, sizeof(double));
    w->dBdT = (double*)calloc(ns, sizeof(double));
    w->Cp = (double*)calloc(ns, sizeof(double));
    w->Ha = (double*)calloc(ns, sizeof(double));
    w->dCpdT = (double*)calloc(ns, sizeof(double));
    w->rhoMvj = (double*)calloc(ns, sizeof(double));
    w->WiByrhoM = (double*)calloc(ns, sizeof(double));
    w->Kinf = (double*)calloc(nr + 1, sizeof(double));
    w->dKinfdT = (double*)calloc(nr + 1, sizeof(double));
    w->Kf = (double*)calloc(nr + 1, sizeof(double));
    w->dKfdT = (double*)calloc(nr + 1, sizeof(double));
    w->M = (double*)calloc(m->nTB + 1, sizeof(double));
    w->Kplog = (double*)calloc(m->nPlog + 1, sizeof(double));
    w->dKplog = (double*)calloc(m->nPlog + 1, sizeof(double));
    w->Jc = (double*)calloc((size_t)n * n, sizeof(double));
    w->Jy = (double*)calloc((size_t)n * n, sizeof(double));
    w->a = (double*)calloc((size_t)n * n, sizeof(double));
    for (int i = 0; i < 16; i++) w->vec[i] = (double*)calloc(n, sizeof(double));
    w->piv = (int*)calloc(n, sizeof(int));
    w->invD = (double*)calloc(n, sizeof(double));
    w->table = (double*)calloc((size_t)12 * n, sizeof(double));
    return w;
}

static void ws_destroy(ws_t* w)
{
    free(w->C); free(w->B); free(w->dBdT); free(w->Cp); free(w->Ha); free(w->dCpdT);
    free(w->rhoMvj); free(w->WiByrhoM); free(w->Kf); free(w->dKfdT); free(w->M);
    free(w->Kinf); free(w->dKinfdT);
    free(w->Kplog); free(w->dKplog); free(w->Jc); free(w->Jy); free(w->a);
    for (int i = 0; i < 16; i++) free(w->vec[i]);
    free(w->piv); free(w->invD); free(w->table);
    free(w);
}

/* ------------------------------------------------------------------------ */
/* thermo: ThermoFunctionI.H                                                 */

static inline const double* coeffs(const orc_mech* m, int i, double Tbranch)
{
    /* setPtrCoeffs (ThermoFunctionI.H:1-31) */
    if (Tbranch < m->TcommonMin) return &m->coef[i * 14];
    if (Tbranch > m->TcommonMax) return &m->coef[i * 14 + 7];
    return (Tbranch < m->Tcommon[i]) ? &m->coef[i * 14] : &m->coef[i * 14 + 7];
}

/* exponent of exp(-G/RT) (ThermoFunctionI.H:539-636): B = a0(lnT-1) + a1 T/2 +
 * a2 T^2/6 + a3 T^3/12 + a4 T^4/20 - a5/T + a6 */
static inline double gibbs_exponent(const double* a, double T, double invT, double logT)
{
    double v = fma(a[4] * 0.05, T, a[3] * (1.0 / 12.0));
    v = fma(v, T, a[2] * (1.0 / 6.0));
    v = fma(v, T, a[1] * 0.5);
    v = fma(v, T, -(a[5] * invT));
    v = v + a[6];
    return fma(a[0], logT - 1.0, v);
}

static inline double cp_of(const double* a, double T, double RuInvW)
{
    double v = fma(a[4], T, a[3]);
    v = fma(v, T, a[2]);
    v = fma(v, T, a[1]);
    v = fma(v, T, a[0]);
    return RuInvW * v;
}

static inline double ha_of(const double* a, double T, double RuInvW)
{
    double v = fma(a[4], T * 0.2, a[3] * 0.25);
    v = fma(v, T, a[2] * (1.0 / 3.0));
    v = fma(v, T, a[1] * 0.5);
    v = fma(v, T, a[0]);
    v = fma(v, T, a[5]);
    return RuInvW * v;
}

/* ------------------------------------------------------------------------ */
/* rate constants shared by RHS and Jacobian                                 */

static void plog_rates(const orc_mech* m, ws_t* w, double p, double logT, double invT, int withDeriv)
{
    /* ReactionRate.C:577-727 / Jacobian.C:798-1000 (uniformPressureRange false) */
    const double logP = log(p);
    for (int i = 0; i < m->nPlog; i++) {
        const int o = m->pOff[i], len = m->pOff[i + 1] - o;
        double lk, dk;
        if (p <= m->pP[o]) {
            lk = m->pLogA[o] + m->pBeta[o] * logT - m->pTa[o] * invT;
            dk = (m->pBeta[o] + m->pTa[o] * invT) * invT;
        } else if (p >= m->pP[o + len - 1]) {
            const int e = o + len - 1;
            lk = m->pLogA[e] + m->pBeta[e] * logT - m->pTa[e] * invT;
            dk = (m->pBeta[e] + m->pTa[e] * invT) * invT;
        } else {
            int idx = 0;
            for (int j = 0; j < len - 1; j++) {
                if (m->pP[o + j] <= p && p <= m->pP[o + j + 1]) { idx = j; break; }
            }
            const int a = o + idx, b = a + 1;
            const double fr = (logP - m->pLogP[a]) / (m->pLogP[b] - m->pLogP[a]);
            lk = m->pLogA[a] + m->pBeta[a] * logT - m->pTa[a] * invT
               + ((m->pLogA[b] - m->pLogA[a]) + (m->pBeta[b] - m->pBeta[a]) * logT
                  - (m->pTa[b] - m->pTa[a]) * invT) * fr;
            dk = invT * (m->pBeta[a] + m->pTa[a] * invT
                         + (m->pBeta[b] - m->pBeta[a] + (m->pTa[b] - m->pTa[a]) * invT) * fr);
        }
        const double k = exp(lk);
        w->Kplog[i] = k;
        if (withDeriv) w->dKplog[i] = k * dk;
    }
}

static void arrhenius_rates(const orc_mech* m, ws_t* w, double logT, double invT, int withDeriv)
{
    /* ReactionRate.C:79-130 (Kf) and Jacobian.C:108-175 (dKf/dT) */
    for (int i = 0; i < m->nr; i++) {
        if (m->kind[i] == FCS_RXN_PLOG) continue;
        if (i < m->nTI) { w->Kf[i] = m->A[i]; w->dKfdT[i] = 0; continue; }
        const double k = m->A[i] * exp(fma(m->beta[i], logT, -(m->Ta[i] * invT)));
        w->Kf[i] = k;
        if (withDeriv) w->dKfdT[i] = k * (fma(m->Ta[i], invT, m->beta[i]) * invT);
        if (IS_FALLOFF(m->kind[i]) || IS_NONEQ(m->kind[i])) {
            /* the second Arrhenius: kInf sits at Ikf[7] + (i - Ikf[4]) in the
             * reference's Kf_ (OptReaction.C:768-772), a non-equilibrium
             * reverse rate at Ikf[9] + (i - Ikf[1]) (OptReaction.C:628-630) */
            const double ki = m->A2[i] * exp(fma(m->beta2[i], logT, -(m->Ta2[i] * invT)));
            w->Kinf[i] = ki;
            if (withDeriv) w->dKinfdT[i] = ki * (fma(m->Ta2[i], invT, m->beta2[i]) * invT);
        }
    }
}

/* Fall-off rate of reaction i from K0 = Kf[i], kInf and M (ReactionRate.C:370-519,
 * pressureReactionFunctionI.H Troe_F_1..3 / SRI_F): Kf = M K0 F / (1 + Pr),
 * Pr = K0 M / kInf, F = 1 (Lindemann), Troe or SRI.  T is the clamped
 * temperature.  With dKfdT / dKfdC (Jacobian.C:426-713, Troe_Jac_1..3,
 * SRI_F_dFdT_dFdPr) also d/dT and d/dM; note that the SRI branch of the
 * reference uses dF/dT at fixed Pr (no dF/dPr dPr/dT term) and the Troe
 * branch the total derivative. */
static double falloff_rate(const orc_mech* m, const ws_t* w, int i, double T, double invT, double* dKfdT,
                           double* dKfdC)
{
    const double K0 = w->Kf[i], Kinf = w->Kinf[i], M = w->M[m->tbRow[i]];
    const double* f = &m->fo[(size_t)i * 5];
    if (m->kind[i] == FCS_RXN_LINDEMANN_FALLOFF) {
        if (!dKfdT) {
            const double Pr = (K0 * M) / Kinf;
            const double N = K0 / (Pr + 1.0);
            return M * N;
        }
        const double invKinf = 1.0 / Kinf;
        const double Pr = (K0 * M) * invKinf;
        const double dPrdT = fma(M, w->dKfdT[i], -(Pr * w->dKinfdT[i])) * invKinf;
        const double tmp = 1.0 / (1.0 + Pr);
        const double dKdT = Pr * w->dKinfdT[i];
        *dKfdT = fma(tmp, dKdT, ((tmp * tmp) * dPrdT) * Kinf);
        *dKfdC = (K0 * tmp) * tmp;
        return M * (tmp * K0);
    }
    const double Pr = K0 * M / Kinf;
    const double logPr = log10(fmax(Pr, SMALL));
    double F, dFdT = 0, dFdPr = 0;
    if (m->kind[i] == FCS_RXN_TROE_FALLOFF) {
        const double alpha = f[0], Ts = f[1], Tss = f[2], Tsss = f[3];
        const double expTTsss = exp(-T * (1.0 / Tsss)), expTTss = exp(-Tss * invT), expTTs = exp(-T * (1.0 / Ts));
        const double Fcent = (1 - alpha) * expTTsss + alpha * expTTs + expTTss;
        const double logFcent = log10(fmax(Fcent, SMALL));
        const double c = -0.4 - 0.67 * logFcent;
        const double n = 0.75 - 1.27 * logFcent;
        const double x1 = n - 0.14 * (logPr + c);
        if (!dKfdT) {
            const double x2 = (logPr + c) / x1;
            const double x3 = 1 + (x2 * x2);
            F = pow(10, logFcent / x3);
        } else {
            const double invx1 = 1.0 / x1;
            const double x2 = (logPr + c) * invx1;
            const double x3 = 1 + (x2 * x2);
            const double invx3 = 1.0 / x3;
            const double x4 = logFcent * invx3;
            F = pow(10, x4);
            const double logTen = log(10.0);
            const double dFcentdT = -(1 - alpha) * (1.0 / Tsss) * expTTsss - alpha * (1.0 / Ts) * expTTs
                                    + Tss * invT * invT * expTTss;
            const double dlogFcentdT = Fcent >= SMALL ? dFcentdT / Fcent / logTen : 0;
            const double dcdT = -0.67 * dlogFcentdT;
            const double dndT = -1.27 * dlogFcentdT;
            const double dx1dT = dndT - 0.14 * dcdT;
            const double dx2dT = (dcdT - x2 * dx1dT) * invx1;
            const double dx3dT = 2 * x2 * dx2dT;
            const double dx4dT = (dlogFcentdT - x4 * dx3dT) * invx3;
            const double dlogPrdPr = Pr >= SMALL ? 1 / (logTen * Pr) : 0;
            const double dx1dPr = -0.14 * dlogPrdPr;
            const double dx2dPr = (dlogPrdPr - x2 * dx1dPr) * invx1;
            const double dx3dPr = 2 * x2 * dx2dPr;
            const double dx4dPr = -x4 * dx3dPr * invx3;
            dFdPr = logTen * F * dx4dPr;
            const double dPrdT = (M * w->dKfdT[i] - Pr * w->dKinfdT[i]) * (1.0 / Kinf);
            dFdT = logTen * F * dx4dT + dFdPr * dPrdT;
        }
    } else {
        const double a = f[0], b = f[1], c = f[2], d = f[3], e = f[4];
        const double X = 1 / (1 + (logPr * logPr));
        if (!dKfdT) {
            const double psi = a * exp(-b / T) + exp(-T / c);
            F = d * pow(psi, X) * pow(T, e);
        } else {
            const double expbT = exp(-b * invT), expTc = exp(-T * (1.0 / c));
            const double psi = a * expbT + expTc;
            F = d * pow(psi, X) * pow(T, e);
            const double dpsidT = a * b / (T * T) * expbT - 1 / c * expTc;
            dFdT = F * (X / psi * dpsidT + e / T);
            const double logTen = log(10.0);
            const double dlogPrdPr = Pr >= SMALL ? 1 / (logTen * Pr) : 0;
            const double dXdPr = -(X * X) * 2 * logPr * dlogPrdPr;
            dFdPr = F * log(psi) * dXdPr;
        }
    }
    const double invOnePlusPr = 1.0 / (1 + Pr);
    if (dKfdT) {
        const double invKinf = 1.0 / Kinf;
        const double dPrdT = (M * w->dKfdT[i] - Pr * w->dKinfdT[i]) * invKinf;
        const double dKdT = Pr * w->dKinfdT[i];
        *dKfdT = F * invOnePlusPr * dKdT + F * invOnePlusPr * invOnePlusPr * dPrdT * Kinf
                 + K0 * invOnePlusPr * dFdT * M;
        *dKfdC = K0 * invOnePlusPr * 1.0 * (F * invOnePlusPr + Pr * dFdPr);
    }
    return M * (invOnePlusPr * F * K0);
}

static void third_body(const orc_mech* m, ws_t* w)
{
    /* M = E.C (ReactionRate.C:131-354) */
    for (int t = 0; t < m->nTB; t++) {
        double s = 0;
        const double* e = &m->eff[(size_t)t * m->ns];
        for (int j = 0; j < m->ns; j++) s += e[j] * w->C[j];
        w->M[t] = s;
    }
}

static inline double prod_sp(const int* sp, int n, const double* C)
{
    double v = 1.0;
    for (int q = 0; q < n; q++) v *= C[sp[q]];
    return v;
}

/* Kc = Kp (Pstd/(Ru T))^dnu, clamped from below (ReactionFunctionI.H RF11..RF33,
 * ChemicalEquilibriumFunctionI.H:14-25) */
static inline double equilibrium(const orc_mech* m, int i, const double* E, double PByRT)
{
    const int* L = &m->lSp[m->lOff[i]];
    const int* R = &m->rSp[m->rOff[i]];
    const int nl = m->lOff[i + 1] - m->lOff[i], nr = m->rOff[i + 1] - m->rOff[i];
    double num = 1.0, den = 1.0;
    for (int q = 0; q < nr; q++) num *= E[R[q]];
    for (int q = 0; q < nl; q++) den *= E[L[q]];
    double Kc = num / den;
    const int dnu = m->dnu[i];
    if (dnu != 0) {
        /* update_Pow_pByRT_SumVki2 table (ChemicalEquilibriumFunctionI.H:14-25);
         * fastPow for the general form (OptReaction.H:1405-1420) */
        double f;
        if (dnu == -2) f = 1 / (PByRT * PByRT);
        else if (dnu == -1) f = 1 / PByRT;
        else if (dnu == 1) f = PByRT;
        else if (dnu == 2) f = PByRT * PByRT;
        else {
            double xx = dnu < 0 ? 1 / PByRT : PByRT;
            f = 1;
            for (int q = dnu; q != 0; q /= 2) { if (q % 2) f *= xx; xx *= xx; }
        }
        Kc = Kc * f;
    }
    const double clamp = (nl > 3 || nr > 3) ? KC_CLAMP_G : KC_CLAMP;
    return Kc > clamp ? Kc : clamp;
}

/* ------------------------------------------------------------------------ */
/* dNdtByV: ReactionRate.C:732-1503                                          */

static void dNdtByV(const orc_mech* m, ws_t* w, double p, double T, double* omega,
                    double* Cp, double* Ha, double TforCpHa, int cpha)
{
    const int ns = m->ns;
    double Tc = T < m->TlowMin ? m->TlowMin : T;
    Tc = Tc > m->ThighMax ? m->ThighMax : Tc;
    const double logT = log(Tc), invT = 1.0 / Tc;
    for (int i = 0; i < ns; i++) {
        const double* a = coeffs(m, i, Tc);
        w->B[i] = exp(gibbs_exponent(a, Tc, invT, logT));
        if (cpha) {
            const double RuInvW = m->invW[i] * RU;
            const double Tp = cpha == 1 ? Tc : TforCpHa;
            Cp[i] = cp_of(a, Tp, RuInvW);
            Ha[i] = ha_of(a, Tp, RuInvW);
        }
    }
    const double PByRT = PSTD / (RU * Tc);
    arrhenius_rates(m, w, logT, invT, 0);
    third_body(m, w);
    for (int i = 0; i < m->nr; i++) {
        if (m->kind[i] == FCS_RXN_THIRD_BODY || m->kind[i] == FCS_RXN_NONEQ_THIRD_BODY) w->Kf[i] *= w->M[m->tbRow[i]];
        else if (IS_FALLOFF(m->kind[i])) w->Kf[i] = falloff_rate(m, w, i, Tc, invT, NULL, NULL);
    }
    if (m->nPlog) plog_rates(m, w, p, logT, invT, 0);
    memset(omega, 0, sizeof(double) * ns);
    for (int i = 0; i < m->nr; i++) {
        const double Kf = (m->kind[i] == FCS_RXN_PLOG) ? w->Kplog[m->plogIdx[i]] : w->Kf[i];
        const int* L = &m->lSp[m->lOff[i]];
        const int* R = &m->rSp[m->rOff[i]];
        const int nl = m->lOff[i + 1] - m->lOff[i], nr = m->rOff[i + 1] - m->rOff[i];
        double Kr = 0;
        if (m->rev[i] == 1) Kr = Kf / equilibrium(m, i, w->B, PByRT);
        else if (m->rev[i] == 2) {
            /* ReactionRate.C:362-367, 540-544: the reverse Arrhenius, times M for third-body */
            Kr = w->Kinf[i];
            if (m->tbRow[i] >= 0) Kr *= w->M[m->tbRow[i]];
        }
        const double q = Kf * prod_sp(L, nl, w->C) - Kr * prod_sp(R, nr, w->C);
        for (int s = 0; s < nl; s++) omega[L[s]] -= q;
        for (int s = 0; s < nr; s++) omega[R[s]] += q;
    }
}

/* FastChemistryModel::derivatives, 7-arg (cpha=1: Cp/Ha at the clamped T,
 * FastChemistryModel.C:194-273) and 6-arg (cpha=2: Cp/Ha from CpHa(T) at the
 * unclamped T, FastChemistryModel.C:340-417).  Clamps Y >= 0 in place. */
static void derivatives(const orc_mech* m, ws_t* w, double p, double* YT, double* dYTdt, int cpha)
{
    const int ns = m->ns;
    const double T = YT[ns];
    for (int i = 0; i < ns; i++) YT[i] = YT[i] > 0 ? YT[i] : 0;
    const double RuTByP = RU * T / p;
    double sum = 0;
    for (int i = 0; i < ns; i++) sum = fma(YT[i] * m->invW[i], RuTByP, sum);
    const double invrhoM = sum;
    const double rhoM = 1.0 / sum;
    for (int i = 0; i < ns; i++) w->C[i] = rhoM * m->invW[i] * YT[i];
    double* Cp = w->Cp;
    double* Ha = w->Ha;
    dNdtByV(m, w, p, T, dYTdt, Cp, Ha, T, cpha);
    double CpM = 0, dTdt = 0;
    for (int i = 0; i < ns; i++) {
        dYTdt[i] = (m->W[i] * invrhoM) * dYTdt[i];
        CpM = fma(YT[i], Cp[i], CpM);
        dTdt = fma(Ha[i], dYTdt[i], dTdt);
    }
    dYTdt[ns] = -dTdt / CpM;
    w->cnt[ORC_RHS]++;
}

/* ------------------------------------------------------------------------ */
/* Jacobian: Jacobian.C:5-1004 + JF11..JF33/JFG + conversion                 */

static void jacobian(const orc_mech* m, ws_t* w, const orc_options* o, double p,
                     double* YT, double* dYTdt, double* J)
{
    const int ns = m->ns, n = m->n;
    for (int i = 0; i < ns; i++) YT[i] = YT[i] > 0 ? YT[i] : 0;
    const double Traw = YT[ns];
    double Tc = Traw < m->TlowMin ? m->TlowMin : Traw;
    Tc = Tc > m->ThighMax ? m->ThighMax : Tc;
    const double logT = log(Tc), invT = 1.0 / Tc;
    double* Jc = w->Jc;
    memset(Jc, 0, sizeof(double) * n * n);
    memset(dYTdt, 0, sizeof(double) * n);

    /* JacobianThermo (ThermoFunctionI.H:33-371), evaluated at the clamped T */
    const double RuTByP = (RU * Tc) / p;
    double rs = 0, MWs = 0;
    for (int i = 0; i < ns; i++) {
        const double* a = coeffs(m, i, Tc);
        rs = fma(RuTByP, YT[i] * m->invW[i], rs);
        MWs = fma(YT[i], m->invW[i], MWs);
        w->dBdT[i] = fma(fma(a[5], invT, a[0]), invT,
                         fma(fma(fma(a[4] * 0.2, Tc, a[3] * 0.25), Tc, a[2] * (1.0 / 3.0)), Tc, a[1] * 0.5));
        w->B[i] = exp(gibbs_exponent(a, Tc, invT, logT));
        const double RuInvW = m->invW[i] * RU;
        w->dCpdT[i] = RuInvW * fma(Tc, fma(Tc, fma(Tc, 4 * a[4], 3 * a[3]), 2 * a[2]), a[1]);
        w->Cp[i] = cp_of(a, Tc, RuInvW);
        w->Ha[i] = ha_of(a, Tc, RuInvW);
    }
    const double MW = 1.0 / MWs;
    const double invRhoM = rs;
    const double rhoM = 1.0 / rs;
    w->rhoM = rhoM;
    w->invT = invT;
    double CpM = 0, dCpMdT = 0;
    for (int i = 0; i < ns; i++) {
        w->rhoMvj[i] = MW * m->invW[i];
        w->WiByrhoM[i] = invRhoM * m->W[i];
        w->C[i] = rhoM * YT[i] * m->invW[i];
        CpM = fma(YT[i], w->Cp[i], CpM);
        dCpMdT = fma(YT[i], w->dCpdT[i], dCpMdT);
    }
    const double PByRT = PSTD / (RU * Tc);
    arrhenius_rates(m, w, logT, invT, 1);
    third_body(m, w);
    if (m->nPlog) plog_rates(m, w, p, logT, invT, 1);
    const double* C = w->C;
    double* omega = dYTdt;
    for (int i = 0; i < m->nr; i++) {
        double Kf, dKfdT, dKfdC = 0;
        int tb = m->tbRow[i];
        if (m->kind[i] == FCS_RXN_PLOG) { Kf = w->Kplog[m->plogIdx[i]]; dKfdT = w->dKplog[m->plogIdx[i]]; }
        else { Kf = w->Kf[i]; dKfdT = w->dKfdT[i]; }
        if (IS_FALLOFF(m->kind[i])) {
            Kf = falloff_rate(m, w, i, Tc, invT, &dKfdT, &dKfdC);
        } else if (tb >= 0) {
            /* Jacobian.C:401-420: dKf/dM = Kf(before M), Kf *= M, dKf/dT *= M */
            dKfdC = Kf;
            Kf *= w->M[tb];
            dKfdT *= w->M[tb];
        }
        const int* L = &m->lSp[m->lOff[i]];
        const int* R = &m->rSp[m->rOff[i]];
        const int nl = m->lOff[i + 1] - m->lOff[i], nr = m->rOff[i + 1] - m->rOff[i];
        double Kr = 0, dKrdT = 0, invKc = 0, dKrdC = 0;
        if (m->rev[i] == 1) {
            /* JF* reversible branch, e.g. JacobianFunctionI.H:1127-1297 */
            const double Kc = equilibrium(m, i, w->B, PByRT);
            const double clamp = (nl > 3 || nr > 3) ? KC_CLAMP_G : KC_CLAMP;
            double sumV = 0;
            for (int q = 0; q < nr; q++) sumV += w->dBdT[R[q]];
            double sumL = 0;
            for (int q = 0; q < nl; q++) sumL += w->dBdT[L[q]];
            sumV -= sumL;
            const double dKcdTByKc = sumV - m->dnu[i] * invT;
            invKc = 1.0 / Kc;
            Kr = Kf * invKc;
            dKrdT = dKfdT * invKc - (Kc > clamp ? Kr * dKcdTByKc : 0);
            dKrdC = dKfdC * invKc;
        } else if (m->rev[i] == 2) {
            /* non-equilibrium overloads of JF*, e.g. JacobianFunctionI.H:100-230:
             * Kr and dKr/dT of the reverse Arrhenius (Jacobian.C:412-422 scale
             * them by M and keep the raw rate as dKr/dM) */
            Kr = w->Kinf[i];
            dKrdT = w->dKinfdT[i];
            if (tb >= 0) {
                dKrdC = Kr;
                Kr *= w->M[tb];
                dKrdT *= w->M[tb];
            }
        }
        if (m->rev[i]) {
            for (int pp = 0; pp < nr; pp++) {
                double d = 1.0;
                for (int q = 0; q < nr; q++) if (q != pp) d *= C[R[q]];
                const double v = -Kr * d;
                const int col = R[pp];
                for (int s = 0; s < nl; s++) Jc[L[s] * n + col] -= v;
                for (int s = 0; s < nr; s++) Jc[R[s] * n + col] += v;
            }
        }
        const double CF = prod_sp(L, nl, C);
        const double CR = prod_sp(R, nr, C);
        const double q = Kf * CF - Kr * CR;
        for (int s = 0; s < nl; s++) omega[L[s]] -= q;
        for (int s = 0; s < nr; s++) omega[R[s]] += q;
        const double dqdT = dKfdT * CF - dKrdT * CR;
        for (int s = 0; s < nl; s++) Jc[L[s] * n + ns] -= dqdT;
        for (int s = 0; s < nr; s++) Jc[R[s] * n + ns] += dqdT;
        for (int pp = 0; pp < nl; pp++) {
            double d = 1.0;
            for (int qq = 0; qq < nl; qq++) if (qq != pp) d *= C[L[qq]];
            const double v = Kf * d;
            const int col = L[pp];
            for (int s = 0; s < nl; s++) Jc[L[s] * n + col] -= v;
            for (int s = 0; s < nr; s++) Jc[R[s] * n + col] += v;
        }
        if (tb >= 0) {
            const double* e = &m->eff[(size_t)tb * ns];
            for (int j = 0; j < ns; j++) {
                const double Wd = (dKfdC * e[j]) * CF - (dKrdC * e[j]) * CR;
                for (int s = 0; s < nl; s++) Jc[L[s] * n + j] -= Wd;
                for (int s = 0; s < nr; s++) Jc[R[s] * n + j] += Wd;
            }
        }
    }

    /* dC/dY conversion */
    double* dYdt_m = w->vec[15];
    for (int i = 0; i < ns; i++) dYdt_m[i] = omega[i] * w->WiByrhoM[i];
    if (o->jacobian == FCS_JACOBIAN_FAST) {
        /* FastddYdtdY (Jacobian.C:4541-4568) */
        for (int i = 0; i < ns; i++)
            for (int j = 0; j < ns; j++)
                J[i * n + j] = w->WiByrhoM[i] * (Jc[i * n + j] * (rhoM * m->invW[j]))
                             + w->rhoMvj[j] * dYdt_m[i];
    } else if (o->conversion_as_written) {
        /* ddYdtdY (Jacobian.C:2814-2858), O(N^3) as written */
        double* arr = w->vec[14];
        for (int j = 0; j < ns; j++) {
            for (int i = 0; i < ns; i++)
                arr[i] = (rhoM * m->invW[i]) * ((i == j ? 1.0 : 0.0) - w->rhoMvj[j] * YT[i]);
            for (int i = 0; i < ns; i++) {
                double s = 0;
                for (int k = 0; k < ns; k++) s += Jc[i * n + k] * arr[k];
                J[i * n + j] = w->WiByrhoM[i] * s + w->rhoMvj[j] * dYdt_m[i];
            }
        }
    } else {
        /* the same conversion as diag scaling + rank-1:
         * sum_k Jc_ik (rho/W_k)(delta_kj - m_j Y_k) = Jc_ij rho/W_j - m_j sum_k Jc_ik C_k */
        for (int i = 0; i < ns; i++) {
            double S = 0;
            for (int k = 0; k < ns; k++) S = fma(Jc[i * n + k], C[k], S);
            for (int j = 0; j < ns; j++)
                J[i * n + j] = w->WiByrhoM[i] * fma(Jc[i * n + j], rhoM * m->invW[j], -(w->rhoMvj[j] * S))
                             + w->rhoMvj[j] * dYdt_m[i];
        }
    }
    /* T column, ddYdtdTP (Jacobian.C:3709-3741) */
    for (int i = 0; i < ns; i++) {
        double v = Jc[i * n + ns];
        for (int j = 0; j < ns; j++) v -= Jc[i * n + j] * C[j] * invT;
        J[i * n + ns] = w->WiByrhoM[i] * v + invT * dYdt_m[i];
        dYTdt[i] = dYdt_m[i];
    }
    /* T row, ddTdtdYT (Jacobian.C:3743-3793) */
    double dTdt = 0;
    for (int i = 0; i < ns; i++) dTdt -= dYTdt[i] * w->Ha[i];
    dTdt /= CpM;
    dYTdt[ns] = dTdt;
    double dd = 0;
    for (int i = 0; i < ns; i++) {
        double v = 0;
        for (int j = 0; j < ns; j++) v -= J[j * n + i] * w->Ha[j];
        v -= w->Cp[i] * dTdt;
        J[ns * n + i] = v / CpM;
        dd -= dYTdt[i] * w->Cp[i] + J[i * n + ns] * w->Ha[i];
    }
    dd -= dTdt * dCpMdT;
    J[ns * n + ns] = dd / CpM;
    w->cnt[ORC_JAC]++;
}

/* ------------------------------------------------------------------------ */
/* LU with 4-row-panel pivoting: LUsolver.C:106-246 (panel), 503-660 (2- and
 * 3-row tails), 3058-3143 (driver); solve LUsolver.C:3145-3171, 4113-4152.   */

static inline void swap_rows(double* a, int n, int r0, int r1)
{
    double* x = &a[(size_t)r0 * n];
    double* y = &a[(size_t)r1 * n];
    for (int j = 0; j < n; j++) { double t = x[j]; x[j] = y[j]; y[j] = t; }
}

/* pivot row for column k at position pos of a panel holding `size` rows */
static int choose_pivot(const double* a, int n, int k, int pos, int size)
{
    const int cand = size - pos;
    if (cand <= 1) return k;
    if (size == 4 && pos == 0) {
        int best = 0; double t = 0;
        for (int c = 0; c < 4; c++) if (t < fabs(a[(size_t)(k + c) * n + k])) { best = c; t = fabs(a[(size_t)(k + c) * n + k]); }
        return k + best;
    }
    if (size == 4 && pos == 1) {
        /* LUsolver.C:169-185: note temp keeps the signed value of row 2 */
        double t = fabs(a[(size_t)k * n + k]); int best = 0;
        if (t < fabs(a[(size_t)(k + 1) * n + k])) { best = 1; t = a[(size_t)(k + 1) * n + k]; }
        if (t < fabs(a[(size_t)(k + 2) * n + k])) { best = 2; }
        return k + best;
    }
    if (size == 3 && pos == 0) {
        int best = 0; double t = 0;
        for (int c = 0; c < 3; c++) if (t < fabs(a[(size_t)(k + c) * n + k])) { best = c; t = fabs(a[(size_t)(k + c) * n + k]); }
        return k + best;
    }
    /* two candidates: swap if |a_kk| < |a_k+1,k| */
    return (fabs(a[(size_t)k * n + k]) < fabs(a[(size_t)(k + 1) * n + k])) ? k + 1 : k;
}

static void lu_decompose(double* a, int n, int* piv, double* invD)
{
    const int rem = n % 4;
    for (int i = 0; i < n; i++) piv[i] = i;
    for (int k = 0; k < n; k++) {
        const int k0 = (k < n - rem) ? (k & ~3) : n - rem;
        const int size = (k < n - rem) ? 4 : rem;
        const int pos = k - k0;
        if (size == 1) {
            invD[k] = 1.0 / a[(size_t)k * n + k];
            continue;
        }
        const int p = choose_pivot(a, n, k, pos, size);
        if (p != k) { swap_rows(a, n, k, p); piv[k] = p; }
        if (a[(size_t)k * n + k] == 0) a[(size_t)k * n + k] = PIV_EPS;
        const double rinv = 1.0 / a[(size_t)k * n + k];
        invD[k] = rinv;
        for (int i = k + 1; i < n; i++) {
            const double l = a[(size_t)i * n + k] * rinv;
            a[(size_t)i * n + k] = l;
            if (l == 0) continue;
            double* ri = &a[(size_t)i * n];
            const double* rk = &a[(size_t)k * n];
            for (int j = k + 1; j < n; j++) ri[j] = fma(-l, rk[j], ri[j]);
        }
    }
}

static void lu_solve(const double* a, int n, const int* piv, const double* invD, double* b)
{
    for (int j = 0; j < n; j++) {
        if (piv[j] != j) { double t = b[piv[j]]; b[piv[j]] = b[j]; b[j] = t; }
    }
    for (int i = 1; i < n; i++) {
        double s = b[i];
        const double* ri = &a[(size_t)i * n];
        for (int j = 0; j < i; j++) s = fma(-ri[j], b[j], s);
        b[i] = s;
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = b[i];
        const double* ri = &a[(size_t)i * n];
        for (int j = i + 1; j < n; j++) s = fma(-ri[j], b[j], s);
        b[i] = s * invD[i];
    }
}

int32_t orc_lu_solve(int32_t n, double* a, int32_t nrhs, double* b, int32_t* piv, double* invD)
{
    lu_decompose(a, n, piv, invD);
    for (int r = 0; r < nrhs; r++) lu_solve(a, n, piv, invD, &b[(size_t)r * n]);
    return FCS_OK;
}

/* ------------------------------------------------------------------------ */
/* Rosenbrock methods                                                        */

typedef struct {
    const orc_mech* m; ws_t* w; const orc_options* o; double p;
} cellctx;

static const double SAFE = 0.9, ALPHA_INC = 0.2, ALPHA_DEC = 0.25, MIN_SCALE = 0.2, MAX_SCALE = 10;

/* OptRodas34::Rodas34Solve (OptRodas34.C:291-882), constants OptRodas34.H:105-149 */
static double rodas34_attempt(cellctx* c, double dx, double invdx, double* y0, double* yTemp)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *k1 = w->vec[0], *k2 = w->vec[1], *k3 = w->vec[2], *k4 = w->vec[3], *k5 = w->vec[4];
    double *dy = w->vec[5], *err = w->vec[6], *dydx = w->vec[7], *dfdx = w->vec[8];
    const double c2 = 0.386, c3 = 0.21, c4 = 0.63;
    const double d1 = 0.25, d2 = -0.1043, d3 = 0.1035, d4 = -0.3620000000000023e-01;
    const double a21 = 0.1544e1, a31 = 0.9466785280815826, a32 = 0.2557011698983284;
    const double a41 = 0.3314825187068521e1, a42 = 0.2896124015972201e1, a43 = 0.9986419139977817;
    const double a51 = 0.1221224509226641e1, a52 = 0.6019134481288629e1, a53 = 0.1253708332932087e2, a54 = -0.6878860361058950;
    const double c21 = -0.56688e1, c31 = -0.2430093356833875e1, c32 = -0.2063599157091915;
    const double c41 = -0.1073529058151375, c42 = -0.9594562251023355e1, c43 = -0.2047028614809616e2;
    const double c51 = 0.7496443313967647e1, c52 = -0.1024680431464352e2, c53 = -0.3399990352819905e2, c54 = 0.1170890893206160e2;
    const double c61 = 0.8083246795921522e1, c62 = -0.7981132988064893e1, c63 = -0.3152159432874371e2, c64 = 0.1631930543123136e2, c65 = -0.6058818238834054e1;
    const double invgamma = 1.0 / 0.25;
    (void)c2; (void)c3; (void)c4;
    double* a = w->a;
    jacobian(m, w, c->o, c->p, y0, dfdx, a);
    for (int i = 0; i < n * n; i++) a[i] = -a[i];
    for (int i = 0; i < n; i++) a[i * n + i] += 1.0 * invdx * invgamma;
    lu_decompose(a, n, w->piv, w->invD);
    w->cnt[ORC_LU]++;
    const double dxd1 = dx * d1 + 1;
    for (int i = 0; i < n; i++) k1[i] = dxd1 * dfdx[i];
    lu_solve(a, n, w->piv, w->invD, k1);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a21, k1[i], y0[i]);
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, e1 = c21 * invdx;
        for (int i = 0; i < n; i++) k2[i] = fma(e1, k1[i], fma(dxd2, dfdx[i], dydx[i]));
    }
    lu_solve(a, n, w->piv, w->invD, k2);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a32, k2[i], fma(a31, k1[i], y0[i]));
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, e1 = c31 * invdx, e2 = c32 * invdx;
        for (int i = 0; i < n; i++) k3[i] = fma(e2, k2[i], fma(e1, k1[i], fma(dxd3, dfdx[i], dydx[i])));
    }
    lu_solve(a, n, w->piv, w->invD, k3);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a43, k3[i], fma(a42, k2[i], fma(a41, k1[i], y0[i])));
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double dxd4 = dx * d4, e1 = c41 * invdx, e2 = c42 * invdx, e3 = c43 * invdx;
        for (int i = 0; i < n; i++)
            k4[i] = fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], fma(dxd4, dfdx[i], dydx[i]))));
    }
    lu_solve(a, n, w->piv, w->invD, k4);
    for (int i = 0; i < n; i++) {
        dy[i] = fma(a54, k4[i], fma(a53, k3[i], fma(a52, k2[i], a51 * k1[i])));
        yTemp[i] = y0[i] + dy[i];
    }
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double e1 = c51 * invdx, e2 = c52 * invdx, e3 = c53 * invdx, e4 = c54 * invdx;
        for (int i = 0; i < n; i++)
            k5[i] = fma(e4, k4[i], fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], dydx[i]))));
    }
    lu_solve(a, n, w->piv, w->invD, k5);
    for (int i = 0; i < n; i++) { dy[i] += k5[i]; yTemp[i] = y0[i] + dy[i]; }
    derivatives(m, w, c->p, yTemp, dydx, 2);
    {
        const double e1 = c61 * invdx, e2 = c62 * invdx, e3 = c63 * invdx, e4 = c64 * invdx, e5 = c65 * invdx;
        for (int i = 0; i < n; i++)
            err[i] = fma(e5, k5[i], fma(e4, k4[i], fma(e3, k3[i], fma(e2, k2[i], fma(e1, k1[i], dydx[i])))));
    }
    lu_solve(a, n, w->piv, w->invD, err);
    w->cnt[ORC_SOLVES] += 6;
    double maxErr = 0;
    for (int i = 0; i < n; i++) {
        yTemp[i] = y0[i] + dy[i] + err[i];
        const double tol = c->o->abs_tol + c->o->rel_tol * fmax(fabs(y0[i]), fabs(yTemp[i]));
        const double e = fabs(err[i]) / tol;
        maxErr = maxErr > e ? maxErr : e;
    }
    return maxErr;
}

/* OptRosenbrock34::Rosenbrock34Solve (OptRosenbrock34.C:281-678), .H:127-158 */
static double ros34_attempt(cellctx* c, double dx, double invdx, double* y0, double* yTemp)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *k1 = w->vec[0], *k2 = w->vec[1], *k3 = w->vec[2], *k4 = w->vec[3];
    double *err = w->vec[6], *dydx = w->vec[7], *dfdx = w->vec[8];
    const double a21 = 2, a31 = 48.0 / 25.0, a32 = 6.0 / 25.0;
    const double c21 = -8, c31 = 372.0 / 25.0, c32 = 12.0 / 5.0;
    const double c41 = -112.0 / 125.0, c42 = -54.0 / 125.0, c43 = -2.0 / 5.0;
    const double b1 = 19.0 / 9.0, b2 = 1.0 / 2.0, b3 = 25.0 / 108.0, b4 = 125.0 / 108.0;
    const double e1 = 34.0 / 108.0, e2 = 7.0 / 36.0, e4 = 125.0 / 108.0;
    const double d1 = 1.0 / 2.0, d2 = -3.0 / 2.0, d3 = 605.0 / 250.0, d4 = 29.0 / 250.0;
    const double invgamma = 1.0 / (1.0 / 2.0);
    double* a = w->a;
    jacobian(m, w, c->o, c->p, y0, dfdx, a);
    for (int i = 0; i < n * n; i++) a[i] = -a[i];
    for (int i = 0; i < n; i++) a[i * n + i] += invdx * invgamma;
    lu_decompose(a, n, w->piv, w->invD);
    w->cnt[ORC_LU]++;
    const double dxd1 = dx * d1 + 1;
    for (int i = 0; i < n; i++) k1[i] = dxd1 * dfdx[i];
    lu_solve(a, n, w->piv, w->invD, k1);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a21, k1[i], y0[i]);
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double dxd2 = dx * d2, f1 = c21 * invdx;
        for (int i = 0; i < n; i++) k2[i] = fma(f1, k1[i], fma(dxd2, dfdx[i], dydx[i]));
    }
    lu_solve(a, n, w->piv, w->invD, k2);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a32, k2[i], fma(a31, k1[i], y0[i]));
    derivatives(m, w, c->p, yTemp, dydx, 1);
    {
        const double dxd3 = dx * d3, f1 = c31 * invdx, f2 = c32 * invdx;
        for (int i = 0; i < n; i++) k3[i] = fma(f2, k2[i], fma(f1, k1[i], fma(dxd3, dfdx[i], dydx[i])));
    }
    lu_solve(a, n, w->piv, w->invD, k3);
    {
        const double dxd4 = dx * d4, f1 = c41 * invdx, f2 = c42 * invdx, f3 = c43 * invdx;
        for (int i = 0; i < n; i++)
            k4[i] = fma(f3, k3[i], fma(f2, k2[i], fma(f1, k1[i], fma(dxd4, dfdx[i], dydx[i]))));
    }
    lu_solve(a, n, w->piv, w->invD, k4);
    w->cnt[ORC_SOLVES] += 4;
    double maxErr = 0;
    for (int i = 0; i < n; i++) {
        yTemp[i] = fma(b4, k4[i], fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i]))));
        err[i] = fma(e4, k4[i], fma(e2, k2[i], e1 * k1[i]));
        const double tol = c->o->abs_tol + c->o->rel_tol * fmax(fabs(y0[i]), fabs(yTemp[i]));
        const double e = fabs(err[i]) / tol;
        maxErr = maxErr > e ? maxErr : e;
    }
    return maxErr;
}

/* OptRodas23::Rodas23Solve (OptRodas23.C:202-315), constants OptRodas23.H:113-126.
 * k2 reuses f(y0); two derivative evaluations per attempt. */
static double rodas23_attempt(cellctx* c, double dx, double invdx, double* y0, double* yTemp)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *k1 = w->vec[0], *k2 = w->vec[1], *k3 = w->vec[2];
    double *dy = w->vec[5], *err = w->vec[6], *dydx = w->vec[7], *dfdx = w->vec[8];
    const double d1 = 1.0 / 2.0, d2 = 3.0 / 2.0, a31 = 2, c21 = 4, c31 = 1, c32 = -1;
    const double c41 = 1, c42 = -1, c43 = -8.0 / 3.0;
    const double invgamma = 1.0 / (1.0 / 2.0);
    double* a = w->a;
    jacobian(m, w, c->o, c->p, y0, dfdx, a);
    for (int i = 0; i < n * n; i++) a[i] = -a[i];
    for (int i = 0; i < n; i++) a[i * n + i] += invdx * invgamma;
    lu_decompose(a, n, w->piv, w->invD);
    w->cnt[ORC_LU]++;
    const double dxd1 = dx * d1, dxd2 = dx * d2;
    for (int i = 0; i < n; i++) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    lu_solve(a, n, w->piv, w->invD, k1);
    for (int i = 0; i < n; i++) k2[i] = fma(dxd2, dfdx[i], dfdx[i]) + c21 * k1[i] / dx;
    lu_solve(a, n, w->piv, w->invD, k2);
    for (int i = 0; i < n; i++) { dy[i] = a31 * k1[i]; yTemp[i] = y0[i] + dy[i]; }
    derivatives(m, w, c->p, yTemp, dydx, 1);
    for (int i = 0; i < n; i++) k3[i] = dydx[i] + fma(c32, k2[i], c31 * k1[i]) / dx;
    lu_solve(a, n, w->piv, w->invD, k3);
    for (int i = 0; i < n; i++) { dy[i] += k3[i]; yTemp[i] = y0[i] + dy[i]; }
    derivatives(m, w, c->p, yTemp, dydx, 1);
    for (int i = 0; i < n; i++) err[i] = dydx[i] + fma(c43, k3[i], fma(c42, k2[i], c41 * k1[i])) / dx;
    lu_solve(a, n, w->piv, w->invD, err);
    w->cnt[ORC_SOLVES] += 4;
    double maxErr = 0;
    for (int i = 0; i < n; i++) {
        yTemp[i] = y0[i] + dy[i] + err[i];
        const double tol = c->o->abs_tol + c->o->rel_tol * fmax(fabs(y0[i]), fabs(yTemp[i]));
        const double e = fabs(err[i]) / tol;
        maxErr = maxErr > e ? maxErr : e;
    }
    return maxErr;
}

/* OptRosenbrock23::Rosenbrock23Solve (OptRosenbrock23.C:208-298), constants
 * OptRosenbrock23.H:116-140.  One derivative evaluation per attempt. */
static double ros23_attempt(cellctx* c, double dx, double invdx, double* y0, double* yTemp)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *k1 = w->vec[0], *k2 = w->vec[1], *k3 = w->vec[2];
    double *err = w->vec[6], *dydx = w->vec[7], *dfdx = w->vec[8];
    const double a21 = 1;
    const double c21 = -1.0156171083877702091975600115545, c31 = 4.0759956452537699824805835358067;
    const double c32 = 9.2076794298330791242156818474003;
    const double b1 = 1, b2 = 6.1697947043828245592553615689730, b3 = -0.4277225654321857332623837380651;
    const double e1 = 0.5, e2 = -2.9079558716805469821718236208017, e3 = 0.2235406989781156962736090927619;
    const double gamma = 0.43586652150845899941601945119356, invgamma = 1.0 / gamma;
    const double d1 = 0.43586652150845899941601945119356, d2 = 0.24291996454816804366592249683314;
    const double d3 = 2.1851380027664058511513169485832;
    double* a = w->a;
    jacobian(m, w, c->o, c->p, y0, dfdx, a);
    for (int i = 0; i < n * n; i++) a[i] = -a[i];
    for (int i = 0; i < n; i++) a[i * n + i] += invdx * invgamma;
    lu_decompose(a, n, w->piv, w->invD);
    w->cnt[ORC_LU]++;
    const double dxd1 = dx * d1, dxd2 = dx * d2, dxd3 = dx * d3;
    for (int i = 0; i < n; i++) k1[i] = fma(dxd1, dfdx[i], dfdx[i]);
    lu_solve(a, n, w->piv, w->invD, k1);
    for (int i = 0; i < n; i++) yTemp[i] = fma(a21, k1[i], y0[i]);
    derivatives(m, w, c->p, yTemp, dydx, 1);
    for (int i = 0; i < n; i++) k2[i] = fma(dxd2, dfdx[i], dydx[i]) + c21 * k1[i] / dx;
    lu_solve(a, n, w->piv, w->invD, k2);
    for (int i = 0; i < n; i++) k3[i] = fma(dxd3, dfdx[i], dydx[i]) + fma(c32, k2[i], c31 * k1[i]) / dx;
    lu_solve(a, n, w->piv, w->invD, k3);
    w->cnt[ORC_SOLVES] += 3;
    double maxErr = 0;
    for (int i = 0; i < n; i++) {
        yTemp[i] = fma(b3, k3[i], fma(b2, k2[i], fma(b1, k1[i], y0[i])));
        err[i] = fma(e3, k3[i], fma(e2, k2[i], e1 * k1[i]));
        const double tol = c->o->abs_tol + c->o->rel_tol * fmax(fabs(y0[i]), fabs(yTemp[i]));
        const double e = fabs(err[i]) / tol;
        maxErr = maxErr > e ? maxErr : e;
    }
    return maxErr;
}

static double rosenbrock_attempt(cellctx* c, double dx, double invdx, double* y0, double* yTemp)
{
    switch (c->o->solver) {
        case FCS_SOLVER_ROSENBROCK34: return ros34_attempt(c, dx, invdx, y0, yTemp);
        case FCS_SOLVER_RODAS23: return rodas23_attempt(c, dx, invdx, y0, yTemp);
        case FCS_SOLVER_ROSENBROCK23: return ros23_attempt(c, dx, invdx, y0, yTemp);
        default: return rodas34_attempt(c, dx, invdx, y0, yTemp);
    }
}

/* ODESolve + adaptiveSolve (OptRodas34.C:123-289, OptRosenbrock34.C:127-279,
 * OptRodas23.C:105-200, OptRosenbrock23.C:105-206: the same controller) */
static int rosenbrock_integrate(cellctx* c, double xEnd, double* dxTryIO, double* y0)
{
    const double ratio = pow(MAX_SCALE / SAFE, -1.0 / ALPHA_INC);
    const double safeMaxScale = SAFE * MAX_SCALE;
    ws_t* w = c->w;
    double* yTemp = w->vec[9];
    const int n = c->m->n;
    double dxTry = *dxTryIO;
    int last = 0;
    double x = 0;
    for (int nStep = 0; nStep < c->o->max_steps; nStep++) {
        const double dxTry0 = dxTry;
        if ((x + dxTry - xEnd) * (x + dxTry - 0.0) > 0) { last = 1; dxTry = xEnd - x; }
        double dx = dxTry, invdx = 1.0 / dx;
        double Err = rosenbrock_attempt(c, dx, invdx, y0, yTemp);
        w->cnt[ORC_ATTEMPTS]++;
        int rejects = 0;
        while (Err > 1) {
            if (++rejects > 100000) return FCS_CELL_DT_UNDERFLOW;
            const double scale = fmax(SAFE * pow(Err, -ALPHA_DEC), MIN_SCALE);
            dx *= scale;
            invdx = 1.0 / dx;
            Err = rosenbrock_attempt(c, dx, invdx, y0, yTemp);
            w->cnt[ORC_ATTEMPTS]++;
        }
        if (!(Err == Err)) return FCS_CELL_NONFINITE;
        w->cnt[ORC_ACCEPTED]++;
        x += dx;
        for (int i = 0; i < n; i++) y0[i] = yTemp[i];
        dxTry = (Err > ratio) ? fmin(fmax(SAFE * pow(Err, -ALPHA_INC), MIN_SCALE), MAX_SCALE) * dx
                              : safeMaxScale * dx;
        if ((x - xEnd) * (xEnd - 0.0) >= 0) {
            if (nStep > 0 && last) dxTry = dxTry0;
            *dxTryIO = dxTry;
            return FCS_CELL_OK;
        }
    }
    return FCS_CELL_MAX_STEPS;
}

/* ------------------------------------------------------------------------ */
/* Seulex: OptSeulex.C:34-94 (setup), 171-260, 262-560, 562-709, 711-734     */

#define KMAXX 12
#define IMAXX (KMAXX + 1)

typedef struct {
    double jacRedo, theta, logTol;
    int kTarg;
    int nSeq[IMAXX];
    double cpu[IMAXX], coeff[IMAXX][IMAXX];
    double dxOpt[IMAXX], temp[IMAXX];
} seulex_t;

static void seulex_init(seulex_t* s, const orc_options* o)
{
    s->jacRedo = fmin(1e-4, o->rel_tol);
    s->theta = 2 * s->jacRedo;
    const double cpuFunc = 1, cpuJac = 5, cpuLU = 1, cpuSolve = 1;
    s->nSeq[0] = 2; s->nSeq[1] = 3;
    for (int i = 2; i < IMAXX; i++) s->nSeq[i] = 2 * s->nSeq[i - 2];
    s->cpu[0] = cpuJac + cpuLU + s->nSeq[0] * (cpuFunc + cpuSolve);
    for (int k = 0; k < KMAXX; k++)
        s->cpu[k + 1] = s->cpu[k] + (s->nSeq[k + 1] - 1) * (cpuFunc + cpuSolve) + cpuLU;
    for (int k = 0; k < IMAXX; k++)
        for (int l = 0; l < k; l++) {
            const double r = (double)s->nSeq[k] / s->nSeq[l];
            s->coeff[k][l] = 1 / (r - 1);
        }
    s->logTol = -log10(o->rel_tol + o->abs_tol) * 0.6 + 0.5;
}

static int seul(cellctx* c, seulex_t* s, double x0, double* y0, double dxTot, int k,
                double* ySeq, double* scale)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *yTemp = w->vec[10], *dy = w->vec[11], *dydx = w->vec[12];
    const int nSteps = s->nSeq[k];
    const double dx = dxTot / nSteps;
    (void)dx;
    const double invdx = nSteps / dxTot;
    double* a = w->a;
    const double* Jy = w->Jy;
    for (int i = 0; i < n * n; i++) a[i] = -Jy[i];
    for (int i = 0; i < n; i++) a[i * n + i] += invdx;
    lu_decompose(a, n, w->piv, w->invD);
    w->cnt[ORC_LU]++;
    (void)x0;
    derivatives(m, w, c->p, y0, dy, 1);
    lu_solve(a, n, w->piv, w->invD, dy);
    w->cnt[ORC_SOLVES]++;
    for (int i = 0; i < n; i++) yTemp[i] = y0[i];
    for (int nn = 1; nn < nSteps; nn++) {
        for (int i = 0; i < n; i++) yTemp[i] += dy[i];
        if (nn == 1 && k <= 1) {
            double dy1 = 0;
            for (int i = 0; i < n; i++) { const double q = dy[i] / scale[i]; dy1 += q * q; }
            dy1 = sqrt(dy1);
            derivatives(m, w, c->p, yTemp, dydx, 1);
            for (int i = 0; i < n; i++) dy[i] = dydx[i] - dy[i] * invdx;
            lu_solve(a, n, w->piv, w->invD, dy);
            w->cnt[ORC_SOLVES]++;
            double dy2 = 0.0;
            for (int i = 0; i < n; i++) {
                if (fabs(dy[i]) > sqrt(VGREAT)) { dy2 = VGREAT; break; }
                const double q = dy[i] / scale[i];
                dy2 += q * q;
            }
            dy2 = sqrt(dy2);
            s->theta = dy2 / fmax(1.0, dy1 + SMALL);
            if (s->theta > 1.0) return 0;
        }
        derivatives(m, w, c->p, yTemp, dy, 1);
        lu_solve(a, n, w->piv, w->invD, dy);
        w->cnt[ORC_SOLVES]++;
    }
    for (int i = 0; i < n; i++) ySeq[i] = yTemp[i] + dy[i];
    return 1;
}

static void extrapolate(seulex_t* s, int k, double* table, int n, double* y)
{
    for (int j = k - 1; j > 0; j--)
        for (int i = 0; i < n; i++)
            table[(j - 1) * n + i] = table[j * n + i] + s->coeff[k][j] * (table[j * n + i] - table[(j - 1) * n + i]);
    for (int i = 0; i < n; i++) y[i] = table[i] + s->coeff[k][0] * (table[i] - y[i]);
}

typedef struct { double dxTry, dxDid; int first, last, reject, prevReject; } sstep_t;

static void seulex_step(cellctx* c, seulex_t* s, double* x, sstep_t* st, double* y)
{
    const orc_mech* m = c->m; ws_t* w = c->w; const int n = m->n;
    double *y0_ = w->vec[0], *ySeq = w->vec[1], *scale = w->vec[2], *k9 = w->vec[3];
    double* table = w->table;
    s->temp[0] = 1e15; /* great */
    double dx = st->dxTry;
    for (int i = 0; i < n; i++) y0_[i] = y[i];
    s->dxOpt[0] = fabs(0.1 * dx);
    if (st->first || st->prevReject) s->theta = 2 * s->jacRedo;
    if (st->first) {
        int kt = (int)s->logTol;
        kt = kt < KMAXX - 1 ? kt : KMAXX - 1;
        s->kTarg = kt > 1 ? kt : 1;
    }
    for (int i = 0; i < n; i++) scale[i] = c->o->abs_tol + c->o->rel_tol * fabs(y[i]);
    int jacUpdated = 0;
    if (s->theta > s->jacRedo) {
        jacobian(m, w, c->o, c->p, y, k9, w->Jy);
        jacUpdated = 1;
    }
    int k = 0;
    double dxNew = fabs(dx);
    int firstk = 1;
    while (firstk || st->reject) {
        dx = dxNew;
        firstk = 0;
        st->reject = 0;
        double errOld = 0;
        for (k = 0; k <= s->kTarg + 1; k++) {
            w->cnt[ORC_ATTEMPTS] += (k == 0);
            int ok = seul(c, s, *x, y0_, dx, k, ySeq, scale);
            if (!ok) { st->reject = 1; dxNew = fabs(dx) * 0.5; break; }
            if (k == 0) for (int i = 0; i < n; i++) y[i] = ySeq[i];
            else for (int i = 0; i < n; i++) table[(k - 1) * n + i] = ySeq[i];
            if (k != 0) {
                extrapolate(s, k, table, n, y);
                double err = 0;
                for (int i = 0; i < n; i++) {
                    scale[i] = c->o->abs_tol + c->o->rel_tol * fabs(y0_[i]);
                    const double q = (y[i] - table[i]) / scale[i];
                    err += q * q;
                }
                err = sqrt(err / n);
                if (err > 1 / SMALL || (k > 1 && err >= errOld)) { st->reject = 1; dxNew = fabs(dx) * 0.5; break; }
                errOld = fmin(4 * err, 1);
                const double expo = 1.0 / (k + 1);
                const double facmin = pow(0.1, expo);
                double fac;
                if (err == 0) fac = 1.0 / facmin;
                else {
                    fac = 0.93 / pow(err / 0.8, expo);
                    fac = fmax(facmin / 4, fmin(1 / facmin, fac));
                }
                s->dxOpt[k] = fabs(dx * fac);
                s->temp[k] = s->cpu[k] / s->dxOpt[k];
                if ((st->first || st->last) && err <= 1.0) break;
                if (k == s->kTarg - 1 && !st->prevReject && !st->first && !st->last) {
                    if (err <= 1.0) break;
                    else if (err > s->nSeq[s->kTarg] * s->nSeq[s->kTarg + 1] * 4.0) {
                        st->reject = 1;
                        s->kTarg = k;
                        if (s->kTarg > 1 && s->temp[k - 1] < 0.7 * s->temp[k]) s->kTarg--;
                        dxNew = s->dxOpt[s->kTarg];
                        break;
                    }
                }
                if (k == s->kTarg) {
                    if (err <= 1.0) break;
                    else if (err > s->nSeq[k + 1] * 2.0) {
                        st->reject = 1;
                        if (s->kTarg > 1 && s->temp[k - 1] < 0.7 * s->temp[k]) s->kTarg--;
                        dxNew = s->dxOpt[s->kTarg];
                        break;
                    }
                }
                if (k == s->kTarg + 1) {
                    if (err > 1.0) {
                        st->reject = 1;
                        if (s->kTarg > 1 && s->temp[s->kTarg - 1] < 0.7 * s->temp[s->kTarg]) s->kTarg--;
                        dxNew = s->dxOpt[s->kTarg];
                    }
                    break;
                }
            }
        }
        if (st->reject) {
            st->prevReject = 1;
            if (!jacUpdated) {
                s->theta = 2.0 * s->jacRedo;
                if (s->theta > s->jacRedo && !jacUpdated) {
                    jacobian(m, w, c->o, c->p, y, k9, w->Jy);
                    jacUpdated = 1;
                }
            }
        }
    }
    st->dxDid = dx;
    *x += dx;
    int kopt;
    if (k == 1) kopt = 2;
    else if (k <= s->kTarg) {
        kopt = k;
        if (s->temp[k - 1] < 0.7 * s->temp[k]) kopt = k - 1;
        else if (s->temp[k] < 0.9 * s->temp[k - 1]) kopt = (k + 1 < KMAXX - 1) ? k + 1 : KMAXX - 1;
    } else {
        kopt = k - 1;
        if (k > 2 && s->temp[k - 2] < 0.7 * s->temp[k - 1]) kopt = k - 2;
        if (s->temp[k] < 0.9 * s->temp[kopt]) kopt = (k < KMAXX - 1) ? k : KMAXX - 1;
    }
    if (st->prevReject) {
        s->kTarg = kopt < k ? kopt : k;
        dxNew = fmin(fabs(dx), s->dxOpt[s->kTarg]);
        st->prevReject = 0;
    } else {
        if (kopt <= k) dxNew = s->dxOpt[kopt];
        else {
            if (k < s->kTarg && s->temp[k] < 0.9 * s->temp[k - 1]) dxNew = s->dxOpt[k] * s->cpu[kopt + 1] / s->cpu[k];
            else dxNew = s->dxOpt[k] * s->cpu[kopt] / s->cpu[k];
        }
        s->kTarg = kopt;
    }
    st->dxTry = dxNew;
}

static int seulex_integrate(cellctx* c, seulex_t* s, double xEnd, double* dxTryIO, double* y0)
{
    ws_t* w = c->w;
    sstep_t st = {*dxTryIO, 0, 1, 0, 0, 0};
    double x = 0;
    for (int nStep = 0; nStep < c->o->max_steps; nStep++) {
        const double dxTry0 = st.dxTry;
        st.reject = 0;
        if ((x + st.dxTry - xEnd) * (x + st.dxTry - 0.0) > 0) { st.last = 1; st.dxTry = xEnd - x; }
        seulex_step(c, s, &x, &st, y0);
        w->cnt[ORC_ACCEPTED]++;
        for (int i = 0; i < c->m->n; i++) if (!(y0[i] == y0[i])) return FCS_CELL_NONFINITE;
        if ((x - xEnd) * (xEnd - 0.0) >= 0) {
            if (nStep > 0 && st.last) st.dxTry = dxTry0;
            *dxTryIO = st.dxTry;
            return FCS_CELL_OK;
        }
        st.first = 0;
        if (st.reject) st.prevReject = 1;
    }
    return FCS_CELL_MAX_STEPS;
}

/* ------------------------------------------------------------------------ */
/* cell loop: FastChemistryModel_transientSolve.H:30-104                     */

typedef struct {
    const orc_mech* m; const orc_options* o;
    int64_t n; double dt; const double* dtc;
    const double *p, *rho0; double *T, *Y, *subDt, *RR; int32_t* status;
    double* dtMinCell;
    volatile int64_t next;
    pthread_mutex_t lock;
    int64_t counters[ORC_NCOUNTERS];
} job_t;

static void* worker(void* arg)
{
    job_t* j = (job_t*)arg;
    const orc_mech* m = j->m;
    const int ns = m->ns, n = m->n;
    ws_t* w = ws_create(m);
    double* y = (double*)malloc(sizeof(double) * n);
    double* Y0 = (double*)malloc(sizeof(double) * ns);
    seulex_t sx;
    seulex_init(&sx, j->o);
    for (;;) {
        int64_t c0 = __atomic_fetch_add((int64_t*)&j->next, 16, __ATOMIC_RELAXED);
        if (c0 >= j->n) break;
        int64_t c1 = c0 + 16 < j->n ? c0 + 16 : j->n;
        for (int64_t c = c0; c < c1; c++) {
            const double deltaT = j->dtc ? j->dtc[c] : j->dt;
            double T = j->T[c];
            j->dtMinCell[c] = 1e300;
            if (!(T > j->o->T_react)) {
                if (j->RR) for (int i = 0; i < ns; i++) j->RR[(size_t)i * j->n + c] = 0;
                if (j->status) j->status[c] = FCS_CELL_SKIPPED;
                continue;
            }
            for (int i = 0; i < ns; i++) Y0[i] = j->Y[(size_t)i * j->n + c];
            double subDt = j->subDt[c];
            cellctx cc = {m, w, j->o, j->p[c]};
            int st = FCS_CELL_OK;
            double timeLeft = deltaT;
            /* Y_ = Y0; solve(p, T, Y_, li, dt, subDt) */
            for (int i = 0; i < ns; i++) y[i] = Y0[i] > 0 ? Y0[i] : 0;
            y[ns] = T;
            while (timeLeft > SMALL) {
                double dtc = timeLeft;
                if (j->o->solver == FCS_SOLVER_SEULEX) st = seulex_integrate(&cc, &sx, dtc, &subDt, y);
                else st = rosenbrock_integrate(&cc, dtc, &subDt, y);
                timeLeft -= dtc;
                if (st != FCS_CELL_OK) break;
            }
            w->cnt[ORC_CELLS]++;
            if (st != FCS_CELL_OK) w->cnt[ORC_FAILED]++;
            for (int i = 0; i < ns; i++) {
                const double Yn = y[i] > 0 ? y[i] : 0.0;
                j->Y[(size_t)i * j->n + c] = Yn;
                if (j->RR) j->RR[(size_t)i * j->n + c] = (Yn * j->rho0[c] - Y0[i] * j->rho0[c]) / deltaT;
            }
            j->T[c] = y[ns];
            j->dtMinCell[c] = subDt;
            j->subDt[c] = subDt < j->o->delta_t_chem_max ? subDt : j->o->delta_t_chem_max;
            if (j->status) j->status[c] = st;
        }
    }
    pthread_mutex_lock(&j->lock);
    for (int i = 0; i < ORC_NCOUNTERS; i++) j->counters[i] += w->cnt[i];
    pthread_mutex_unlock(&j->lock);
    free(y); free(Y0);
    ws_destroy(w);
    return NULL;
}

void orc_default_options(orc_options* o)
{
    o->solver = FCS_SOLVER_RODAS34;
    o->jacobian = FCS_JACOBIAN_EXACT;
    o->conversion_as_written = 0;
    o->max_steps = 10000;
    o->abs_tol = 1e-8;
    o->rel_tol = 1e-4;
    o->T_react = 0.0;
    o->delta_t_chem_max = 1e300;
    o->n_threads = 1;
}

int32_t orc_integrate(const orc_mech* m, const orc_options* o, int64_t n_cells,
                      double delta_t, const double* dtc, const double* p, const double* rho0,
                      double* T, double* Y, double* sub_dt, double* RR, int32_t* cell_status,
                      double* delta_t_min, int64_t* counters)
{
    job_t j;
    memset(&j, 0, sizeof(j));
    j.m = m; j.o = o; j.n = n_cells; j.dt = delta_t; j.dtc = dtc;
    j.p = p; j.rho0 = rho0; j.T = T; j.Y = Y; j.subDt = sub_dt; j.RR = RR; j.status = cell_status;
    j.dtMinCell = (double*)malloc(sizeof(double) * (n_cells > 0 ? n_cells : 1));
    pthread_mutex_init(&j.lock, NULL);
    int nt = o->n_threads > 0 ? o->n_threads : 1;
    if (nt == 1) worker(&j);
    else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
        for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, worker, &j);
        for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
        free(th);
    }
    pthread_mutex_destroy(&j.lock);
    double dmin = 1e15; /* great */
    for (int64_t c = 0; c < n_cells; c++) if (j.dtMinCell[c] < dmin) dmin = j.dtMinCell[c];
    free(j.dtMinCell);
    const double dtref = dtc ? dtc[0] : delta_t;
    if (delta_t_min) *delta_t_min = dmin < 2 * dtref ? dmin : 2 * dtref;
    if (counters) for (int i = 0; i < ORC_NCOUNTERS; i++) counters[i] = j.counters[i];
    return j.counters[ORC_FAILED] ? FCS_ERR_CELLS : FCS_OK;
}

int32_t orc_rhs(const orc_mech* m, int64_t n_cells, const double* p, const double* T,
                const double* Y, double* dydt)
{
    ws_t* w = ws_create(m);
    const int ns = m->ns, n = m->n;
    double* y = (double*)malloc(sizeof(double) * n);
    double* f = (double*)malloc(sizeof(double) * n);
    for (int64_t c = 0; c < n_cells; c++) {
        for (int i = 0; i < ns; i++) y[i] = Y[(size_t)i * n_cells + c];
        y[ns] = T[c];
        derivatives(m, w, p[c], y, f, 1);
        for (int i = 0; i < n; i++) dydt[(size_t)i * n_cells + c] = f[i];
    }
    free(y); free(f);
    ws_destroy(w);
    return FCS_OK;
}

int32_t orc_jacobian(const orc_mech* m, const orc_options* o, int64_t n_cells,
                     const double* p, const double* T, const double* Y, double* J, double* dydt)
{
    ws_t* w = ws_create(m);
    const int ns = m->ns, n = m->n;
    double* y = (double*)malloc(sizeof(double) * n);
    double* f = (double*)malloc(sizeof(double) * n);
    for (int64_t c = 0; c < n_cells; c++) {
        for (int i = 0; i < ns; i++) y[i] = Y[(size_t)i * n_cells + c];
        y[ns] = T[c];
        jacobian(m, w, o, p[c], y, f, &J[(size_t)c * n * n]);
        for (int i = 0; i < n; i++) dydt[(size_t)i * n_cells + c] = f[i];
    }
    free(y); free(f);
    ws_destroy(w);
    return FCS_OK;
}

/* FastChemistryModel::calculate (FastChemistryModel.C:715-755): c_i = rho Y_i / W_i
 * (no clamp), RR_i = dNdtByV_i W_i; Qdot = -sum Hf_i RR_i (FastChemistryModel.C:656-685)
 * with Hf the janaf enthalpy at 298.15 K. */
/* OptReaction::fastPow (OptReaction.H:1405-1420) */
static double fast_pow(double x, int order)
{
    double xx = order < 0 ? 1 / x : x;
    double y = 1;
    for (int i = order; i != 0; i /= 2) {
        if (i % 2) y *= xx;
        xx *= xx;
    }
    return y;
}

/* FastChemistryModel::tc (FastChemistryModel.C:589-651) over OptReaction::Tc
 * (Tc.C:3-834): per reaction wf = n_products Kf CF, wr = n_reactants Kr CR,
 * tc = sum(w) / sum(w^2) * sum(c), c = rho Y / W (Y not clamped). */
int32_t orc_tc(const orc_mech* m, int64_t n_cells, const double* p, const double* T, const double* rho,
               const double* Y, double* tc)
{
    ws_t* w = ws_create(m);
    const int ns = m->ns;
    for (int64_t c = 0; c < n_cells; c++) {
        double sumc = 0;
        for (int i = 0; i < ns; i++) {
            w->C[i] = rho[c] * Y[(size_t)i * n_cells + c] / m->W[i];
            sumc += w->C[i];
        }
        double Tc = T[c] < m->TlowMin ? m->TlowMin : T[c];
        Tc = Tc > m->ThighMax ? m->ThighMax : Tc;
        const double logT = log(Tc), invT = 1.0 / Tc;
        for (int i = 0; i < ns; i++) w->B[i] = exp(gibbs_exponent(coeffs(m, i, Tc), Tc, invT, logT));
        const double PByRT = PSTD / (RU * Tc);
        arrhenius_rates(m, w, logT, invT, 0);
        third_body(m, w);
        for (int i = 0; i < m->nr; i++) {
            if (m->kind[i] == FCS_RXN_THIRD_BODY || m->kind[i] == FCS_RXN_NONEQ_THIRD_BODY) w->Kf[i] *= w->M[m->tbRow[i]];
            else if (IS_FALLOFF(m->kind[i])) w->Kf[i] = falloff_rate(m, w, i, Tc, invT, NULL, NULL);
        }
        if (m->nPlog) plog_rates(m, w, p[c], logT, invT, 0);
        double sumW = 0, sumWR = 0;
        for (int i = 0; i < m->nr; i++) {
            const double Kf = (m->kind[i] == FCS_RXN_PLOG) ? w->Kplog[m->plogIdx[i]] : w->Kf[i];
            const int* L = &m->lSp[m->lOff[i]];
            const int* R = &m->rSp[m->rOff[i]];
            const int nl = m->lOff[i + 1] - m->lOff[i], nr = m->rOff[i + 1] - m->rOff[i];
            double Kr = 0, Kp = 1.0;
            /* Tc.C:578-600: the reverse rate only through Kc; a non-equilibrium
             * reaction counts with its forward rate alone */
            if (m->rev[i] == 1) {
                for (int q = 0; q < nl; q++) Kp = Kp / w->B[L[q]];
                for (int q = 0; q < nr; q++) Kp = Kp * w->B[R[q]];
                double Kc = Kp * fast_pow(PByRT, nr - nl);
                Kc = Kc > KC_CLAMP_G ? Kc : KC_CLAMP_G;
                Kr = Kf / Kc;
            }
            const double wf = nr * (Kf * prod_sp(L, nl, w->C));
            const double wr = nl * (Kr * prod_sp(R, nr, w->C));
            sumW += wf;
            sumWR += wf * wf;
            sumW += wr;
            sumWR += wr * wr;
        }
        tc[c] = sumWR == 0 ? 1e300 : sumW / sumWR * sumc;
    }
    ws_destroy(w);
    return FCS_OK;
}

int32_t orc_rates(const orc_mech* m, int64_t n_cells, const double* p, const double* T, const double* rho,
                  const double* Y, double* RR, double* Qdot)
{
    ws_t* w = ws_create(m);
    const int ns = m->ns;
    double* om = (double*)malloc(sizeof(double) * ns);
    for (int64_t c = 0; c < n_cells; c++) {
        for (int i = 0; i < ns; i++) w->C[i] = rho[c] * Y[(size_t)i * n_cells + c] / m->W[i];
        dNdtByV(m, w, p[c], T[c], om, w->Cp, w->Ha, T[c], 1);
        double q = 0;
        for (int i = 0; i < ns; i++) {
            const double rr = om[i] * m->W[i];
            RR[(size_t)i * n_cells + c] = rr;
            const double* a = (298.15 < m->Tcommon[i]) ? &m->coef[i * 14] : &m->coef[i * 14 + 7];
            const double t = 298.15;
            const double hf = RU * m->invW[i] * (((((a[4] / 5 * t + a[3] / 4) * t + a[2] / 3) * t + a[1] / 2) * t + a[0]) * t + a[5]);
            q -= hf * rr;
        }
        if (Qdot) Qdot[c] = q;
    }
    free(om);
    ws_destroy(w);
    return FCS_OK;
}
