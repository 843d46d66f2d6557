/*
 * omd_oracle.c -- CPU FP64 restatement of the Object-MD force path.
 * TEST INFRASTRUCTURE ONLY (see omd_oracle.h); compile with
 * -ffp-contract=off so the FP64 operation order matches the reference on
 * every host architecture.
 */
#include "omd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ tables */

void oc_table_coef(oc_table* t) {
    /* treader.cpp:37-64, same operation order. */
    int nd = t->n;
    int n = nd - 2;
    double* b = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* d = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* S = (double*)malloc(sizeof(double) * nd);
    double dr = t->dr;
    for (int i = 1; i < n + 1; i++) d[i - 1] = t->d[i + 1] - 2.0 * t->d[i] + t->d[i - 1];
    for (int i = 1; i < n - 1; i++) b[i] = 4.0;
    b[0] = b[n - 1] = 5.0;
    for (int k = 1; k < n; k++) {
        double m = 1.0 / b[k - 1];
        b[k] -= m;
        d[k] -= m * d[k - 1];
    }
    S[n + 1] = S[n] = d[n - 1] / b[n - 1];
    for (int k = n - 2; k >= 0; k--) S[k + 1] = (d[k] - 1.0 * S[k + 2]) / b[k];
    S[0] = S[1];
    for (int i = 0; i < nd; i++) t->a[i] = t->b[i] = t->c[i] = 0.0;
    for (int i = 0; i < nd - 1; i++) {
        t->a[i] = (S[i + 1] - S[i]) / dr / dr / dr;
        t->b[i] = 3.0 * S[i] / dr / dr;
        t->c[i] = (t->d[i + 1] - t->d[i] - 2.0 * S[i] - S[i + 1]) / dr;
    }
    free(b);
    free(d);
    free(S);
}

double oc_table_max_range(const oc_table* t) { return t->off + (double)(t->n - 1) * t->dr; }

int oc_table_read(const oc_table* t, double r, double* val, double* dval) {
    /* treader.cpp:193-229 */
    double rval = r - t->off;
    int x = (int)(rval / t->dr);
    double dx = rval - (double)x * t->dr;
    if (x > t->n - 1) {
        if (t->allow_hi) {
            *val = *dval = t->out_hi;
            return 0;
        }
        return -1;
    }
    if (x < -1) {
        if (t->allow_lo) {
            *val = *dval = t->out_lo;
            return 0;
        }
        return -1;
    }
    if (x == t->n - 1) {
        dx += t->dr;
        x--;
    }
    if (x == -1) x = 0;
    double v = (t->d[x] + dx * (t->c[x] + dx * (t->b[x] + dx * t->a[x])));
    double dv = (t->c[x] + dx * (2.0 * t->b[x] + 3.0 * dx * t->a[x]));
    if (t->rmult) {
        v /= r;
        dv = (dv - v) / r;
    }
    *val = v;
    *dval = dv;
    return 0;
}

/* ------------------------------------------------------------- neighbours */

static void shift_vec(const oc_box* box, int code, double s[3]) {
    int sx = code % 3 - 1, sy = (code / 3) % 3 - 1, sz = code / 9 - 1;
    s[0] = sx == 0 ? 0.0 : (sx > 0 ? (box->hi[0] - box->lo[0]) : -(box->hi[0] - box->lo[0]));
    s[1] = sy == 0 ? 0.0 : (sy > 0 ? (box->hi[1] - box->lo[1]) : -(box->hi[1] - box->lo[1]));
    s[2] = sz == 0 ? 0.0 : (sz > 0 ? (box->hi[2] - box->lo[2]) : -(box->hi[2] - box->lo[2]));
}

/* dx = x_i - (x_j + s): the ghost image coordinate is rounded first
   (comhandler.cpp:349-355), then differenced (gadget.cpp:140-145). */
static double pair_dist2(const double* xi, const double* xj, const double s[3], double d[3]) {
    double gx = xj[0] + s[0], gy = xj[1] + s[1], gz = xj[2] + s[2];
    d[0] = xi[0] - gx;
    d[1] = xi[1] - gy;
    d[2] = xi[2] - gz;
    return (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

typedef struct {
    int j, code;
} oc_tuple;

static int cmp_tuple(const void* a, const void* b) {
    const oc_tuple* x = (const oc_tuple*)a;
    const oc_tuple* y = (const oc_tuple*)b;
    if (x->j != y->j) return x->j < y->j ? -1 : 1;
    return x->code < y->code ? -1 : (x->code > y->code);
}

/* The sorted row of atom i: every (j, image) with r^2 <= rsq over the
   linked cells (VerletList.cpp:76-199 with the ghost images of
   comhandler.cpp:288-377).  Returns its length; *row grows as needed. */
static int atom_row(const oc_box* box, const double* x, double rsq, const int* nc, const int* cell, const int* head,
                    const int* next, int i, oc_tuple** row, int* rowcap) {
    int ci[3] = {cell[i] % nc[0], (cell[i] / nc[0]) % nc[1], cell[i] / (nc[0] * nc[1])};
    int cand_c[3][64], cand_s[3][64], ncand[3];
    for (int d = 0; d < 3; d++) {
        ncand[d] = 0;
        if (box->periodic[d]) {
            if (nc[d] >= 3) {
                for (int o = -1; o <= 1; o++) {
                    int c = ci[d] + o, s = 0;
                    if (c < 0) {
                        c += nc[d];
                        s = -1;
                    } else if (c >= nc[d]) {
                        c -= nc[d];
                        s = 1;
                    }
                    cand_c[d][ncand[d]] = c;
                    cand_s[d][ncand[d]++] = s;
                }
            } else {
                for (int c = 0; c < nc[d]; c++)
                    for (int s = -1; s <= 1; s++) {
                        cand_c[d][ncand[d]] = c;
                        cand_s[d][ncand[d]++] = s;
                    }
            }
        } else {
            for (int o = -1; o <= 1; o++) {
                int c = ci[d] + o;
                if (c < 0 || c >= nc[d]) continue;
                cand_c[d][ncand[d]] = c;
                cand_s[d][ncand[d]++] = 0;
            }
        }
    }
    int nrow = 0;
    for (int a = 0; a < ncand[2]; a++)
        for (int b = 0; b < ncand[1]; b++)
            for (int c = 0; c < ncand[0]; c++) {
                int code = (cand_s[0][c] + 1) + 3 * (cand_s[1][b] + 1) + 9 * (cand_s[2][a] + 1);
                double s[3];
                shift_vec(box, code, s);
                long cc = ((long)cand_c[2][a] * nc[1] + cand_c[1][b]) * nc[0] + cand_c[0][c];
                for (int j = head[cc]; j >= 0; j = next[j]) {
                    if (j == i && code == 13) continue;
                    double dd[3];
                    double r2 = pair_dist2(x + 3 * i, x + 3 * j, s, dd);
                    if (r2 <= rsq) {
                        if (nrow == *rowcap) {
                            *rowcap *= 2;
                            *row = (oc_tuple*)realloc(*row, sizeof(oc_tuple) * (*rowcap));
                        }
                        (*row)[nrow].j = j;
                        (*row)[nrow].code = code;
                        nrow++;
                    }
                }
            }
    qsort(*row, nrow, sizeof(oc_tuple), cmp_tuple);
    return nrow;
}

long oc_neighbors(const oc_box* box, int n, const double* x, double rv, int* offsets, int* nbr_j, int* nbr_code,
                  long cap) {
    double rsq = rv * rv;
    int nc[3];
    double org[3], h[3];
    for (int d = 0; d < 3; d++) {
        if (box->periodic[d]) {
            double L = box->hi[d] - box->lo[d];
            org[d] = box->lo[d];
            nc[d] = (int)(L / rv);
            if (nc[d] < 1) nc[d] = 1;
            h[d] = L / nc[d];
        } else {
            double mn = 1e300, mx = -1e300;
            for (int i = 0; i < n; i++) {
                if (x[3 * i + d] < mn) mn = x[3 * i + d];
                if (x[3 * i + d] > mx) mx = x[3 * i + d];
            }
            org[d] = mn;
            nc[d] = (int)((mx - mn) / rv);
            if (nc[d] < 1) nc[d] = 1;
            h[d] = (mx - mn) / nc[d];
            if (h[d] <= 0) h[d] = 1.0;
        }
    }
    long ncell = (long)nc[0] * nc[1] * nc[2];
    int* cell = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    int* head = (int*)malloc(sizeof(int) * ncell);
    int* next = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (long c = 0; c < ncell; c++) head[c] = -1;
    for (int i = n - 1; i >= 0; i--) {
        int ci[3];
        for (int d = 0; d < 3; d++) {
            if (box->periodic[d] && (x[3 * i + d] < box->lo[d] || x[3 * i + d] >= box->hi[d])) {
                free(cell);
                free(head);
                free(next);
                return -2; /* periodic positions must be wrapped first */
            }
            int c = (int)floor((x[3 * i + d] - org[d]) / h[d]);
            if (c < 0) c = 0;
            if (c >= nc[d]) c = nc[d] - 1;
            ci[d] = c;
        }
        cell[i] = (ci[2] * nc[1] + ci[1]) * nc[0] + ci[0];
        next[i] = head[cell[i]];
        head[cell[i]] = i;
    }
    long count = 0;
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    if (nth <= 1) {
        oc_tuple* row = (oc_tuple*)malloc(sizeof(oc_tuple) * 4096);
        int rowcap = 4096;
        for (int i = 0; i < n; i++) {
            int nrow = atom_row(box, x, rsq, nc, cell, head, next, i, &row, &rowcap);
            offsets[i] = (int)count;
            for (int k = 0; k < nrow; k++) {
                if (count >= cap) {
                    free(row);
                    free(cell);
                    free(head);
                    free(next);
                    return -1;
                }
                nbr_j[count] = row[k].j;
                nbr_code[count] = row[k].code;
                count++;
            }
        }
        offsets[n] = (int)count;
        free(row);
    } else {
        /* threads (timing runs): row lengths, their prefix, then the rows */
        int* len = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
#pragma omp parallel
        {
            int rowcap = 4096;
            oc_tuple* row = (oc_tuple*)malloc(sizeof(oc_tuple) * rowcap);
#pragma omp for schedule(static)
            for (int i = 0; i < n; i++) len[i] = atom_row(box, x, rsq, nc, cell, head, next, i, &row, &rowcap);
            free(row);
        }
        for (int i = 0; i < n; i++) {
            offsets[i] = (int)count;
            count += len[i];
        }
        offsets[n] = (int)count;
        free(len);
        if (count > cap) {
            free(cell);
            free(head);
            free(next);
            return -1;
        }
#pragma omp parallel
        {
            int rowcap = 4096;
            oc_tuple* row = (oc_tuple*)malloc(sizeof(oc_tuple) * rowcap);
#pragma omp for schedule(static)
            for (int i = 0; i < n; i++) {
                int nrow = atom_row(box, x, rsq, nc, cell, head, next, i, &row, &rowcap);
                for (int k = 0; k < nrow; k++) {
                    nbr_j[offsets[i] + k] = row[k].j;
                    nbr_code[offsets[i] + k] = row[k].code;
                }
            }
            free(row);
        }
    }
    free(cell);
    free(head);
    free(next);
    return count;
}

/* ------------------------------------------------------------------ forces */

static void zero3(int n, double* f, double* e, double* vir) {
    memset(f, 0, sizeof(double) * 3 * n);
    memset(e, 0, sizeof(double) * n);
    memset(vir, 0, sizeof(double) * n);
}

int oc_eam(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j, const int* nbr_code,
           const oc_table* phi, const oc_table* edens, const oc_table* embed, double* f, double* e, double* vir,
           double* rho) {
    double rc_phi = oc_table_max_range(phi), rc_rho = oc_table_max_range(edens);
    double* fp = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    int bad = 0;
    zero3(n, f, e, vir);
    /* density pass: team.cpp:81-92, R <= CutRadius of the density table
       (every atom's sum is its own: threads change nothing but the time) */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++) {
        double acc = 0.0;
        for (int k = offsets[i]; k < offsets[i + 1]; k++) {
            double s[3], d[3];
            shift_vec(box, nbr_code[k], s);
            double R = sqrt(pair_dist2(x + 3 * i, x + 3 * nbr_j[k], s, d));
            if (R <= rc_rho) {
                double v, dv;
                if (oc_table_read(edens, R, &v, &dv)) {
                    bad = 1;
                    break;
                }
                acc += v;
            }
        }
        rho[i] = acc;
        double Fv = 0.0, Fd = 0.0;
        if (oc_table_read(embed, acc, &Fv, &Fd)) bad = 1;
        fp[i] = Fd;
        e[i] = Fv; /* team.cpp:135-145 */
    }
    if (bad) {
        free(fp);
        return -1;
    }
    /* force pass: team.cpp:224-237 and forcekernel.h:92-110 */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++) {
        for (int k = offsets[i]; k < offsets[i + 1]; k++) {
            int j = nbr_j[k];
            double s[3], d[3];
            shift_vec(box, nbr_code[k], s);
            double r2 = pair_dist2(x + 3 * i, x + 3 * j, s, d);
            double R = sqrt(r2);
            if (R <= rc_phi) {
                double p, dp, rv_, drho;
                if (oc_table_read(phi, R, &p, &dp)) {
                    bad = 1;
                    break;
                }
                drho = 0.0;
                if (!(R > rc_rho)) {
                    if (oc_table_read(edens, R, &rv_, &drho)) {
                        bad = 1;
                        break;
                    }
                }
                double fr = -(fp[i] * drho + fp[j] * drho + dp) / R;
                f[3 * i + 0] += d[0] * fr;
                f[3 * i + 1] += d[1] * fr;
                f[3 * i + 2] += d[2] * fr;
                e[i] += 0.5 * p;
                vir[i] += d[0] * fr * d[0] + d[1] * fr * d[1] + d[2] * fr * d[2];
            }
        }
    }
    free(fp);
    return bad ? -1 : 0;
}

int oc_pair_table_typed(const oc_box* box, int n, const double* x, const int* type, int ta, int tb,
                        const int* offsets, const int* nbr_j, const int* nbr_code, const oc_table* phi, double* f,
                        double* e, double* vir) {
    double rc = oc_table_max_range(phi);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++) {
        for (int k = offsets[i]; k < offsets[i + 1]; k++) {
            int j = nbr_j[k];
            if (type) {
                int a = type[i], b = type[j];
                if (!((a == ta && b == tb) || (a == tb && b == ta))) continue;
            }
            double s[3], d[3];
            shift_vec(box, nbr_code[k], s);
            double r = sqrt(pair_dist2(x + 3 * i, x + 3 * j, s, d));
            if (r < rc) {
                double p, dp;
                if (oc_table_read(phi, r, &p, &dp)) {
                    bad = 1;
                    break;
                }
                double fr = -dp / r;
                f[3 * i + 0] += d[0] * fr;
                f[3 * i + 1] += d[1] * fr;
                f[3 * i + 2] += d[2] * fr;
                e[i] += 0.5 * p;
                vir[i] += d[0] * fr * d[0] + d[1] * fr * d[1] + d[2] * fr * d[2];
            }
        }
    }
    return bad ? -1 : 0;
}

int oc_zbl(const oc_box* box, int n, const double* x, const int* type, int ta, int tb, double z1, double z2,
           double rc, double width, const int* offsets, const int* nbr_j, const int* nbr_code, double* f, double* e,
           double* vir) {
    /* sw.cpp:84-91 */
    const double znor = 0.468521928 / (pow(z1, 0.23) + pow(z2, 0.23));
    const double zc = 14.39964415 * z1 * z2;
    const double ze[4] = {3.2000 / znor, 0.9423 / znor, 0.4029 / znor, 0.2016 / znor};
    const double cf[4] = {0.1818, 0.5099, 0.2802, 0.02817};
    const double rsw = rc - width;
    for (int i = 0; i < n; i++) {
        for (int k = offsets[i]; k < offsets[i + 1]; k++) {
            int j = nbr_j[k];
            int a = type[i], b = type[j];
            if (!((a == ta && b == tb) || (a == tb && b == ta))) continue;
            double s[3], d[3];
            shift_vec(box, nbr_code[k], s);
            double r = sqrt(pair_dist2(x + 3 * i, x + 3 * j, s, d));
            if (!(r < rc)) continue;
            /* sw.cpp:121-134: fpot and fr = -dfpot/dr / r */
            double fex[4], sum = 0.0, dsum = 0.0;
            for (int q = 0; q < 4; q++) {
                fex[q] = cf[q] * exp(-ze[q] * r);
                sum += fex[q];
                dsum += (1.0 / r + ze[q]) * fex[q];
            }
            double phi = sum * zc / r;
            double dphi = -dsum * zc / r; /* d phi / dr */
            double S = 1.0, dS = 0.0;
            if (r > rsw) {
                double t = (r - rsw) / width;
                S = 1.0 - t * t * t * (10.0 - 15.0 * t + 6.0 * t * t);
                dS = -30.0 * t * t * (1.0 - t) * (1.0 - t) / width;
            }
            double v = phi * S, dv = dphi * S + phi * dS;
            double fr = -dv / r;
            f[3 * i + 0] += d[0] * fr;
            f[3 * i + 1] += d[1] * fr;
            f[3 * i + 2] += d[2] * fr;
            e[i] += 0.5 * v;
            vir[i] += fr * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        }
    }
    return 0;
}

int oc_pair_table(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j,
                  const int* nbr_code, const oc_table* phi, double* f, double* e, double* vir) {
    zero3(n, f, e, vir);
    return oc_pair_table_typed(box, n, x, 0, 0, 0, offsets, nbr_j, nbr_code, phi, f, e, vir);
}

/* ---------------------------------------------------------------- SW */

typedef struct {
    double rc, c1, c2, c3, c4, c5, c6, c7, c8, c9, c10, zc, ze0, ze1, ze2, ze3;
} sw_const;

static void sw_constants(const oc_sw_param* p, sw_const* k) {
    /* sw.cpp:65-91 */
    k->rc = p->a * p->sigma;
    k->c1 = p->A * p->eps * p->p * p->B * pow(p->sigma, p->p);
    k->c2 = p->A * p->eps * p->q * pow(p->sigma, p->q);
    k->c3 = p->A * p->eps * p->B * pow(p->sigma, p->p + 1.0);
    k->c4 = p->A * p->eps * pow(p->sigma, p->q + 1.0);
    k->c5 = p->A * p->eps * p->B * pow(p->sigma, p->p);
    k->c6 = p->A * p->eps * pow(p->sigma, p->q);
    k->c7 = p->sigma * p->gamma;
    k->c8 = p->lambda * p->eps;
    k->c9 = 2.0 * p->lambda * p->eps;
    k->c10 = 1.0 / p->icos0;
    double znor = 0.468521928 / (pow(p->z1, 0.23) + pow(p->z2, 0.23));
    k->zc = 14.39964415 * p->z1 * p->z2;
    k->ze0 = 3.2000 / znor;
    k->ze1 = 0.9423 / znor;
    k->ze2 = 0.4029 / znor;
    k->ze3 = 0.2016 / znor;
}

/* Two-body part for the pair (i, j) with d = x_i - x_j: returns the force
   factor fr (force on i = fr * d) and the energy share of each atom. */
static void sw_two_body(const oc_sw_param* p, const sw_const* k, double r, double* fr, double* half_e) {
    if (p->usezbl && r < p->sx0) {
        /* sw.cpp:118-146 */
        double fex0 = 0.1818 * exp(-k->ze0 * r);
        double fex1 = 0.5099 * exp(-k->ze1 * r);
        double fex2 = 0.2802 * exp(-k->ze2 * r);
        double fex3 = 0.02817 * exp(-k->ze3 * r);
        double fpot = (fex0 + fex1 + fex2 + fex3) * k->zc / r;
        *fr = ((1.0 / r + k->ze0) * fex0 + (1.0 / r + k->ze1) * fex1 + (1.0 / r + k->ze2) * fex2 +
               (1.0 / r + k->ze3) * fex3) *
              k->zc / (r * r);
        *half_e = fpot * 0.5;
    } else if (p->usezbl && r < p->sx1) {
        /* sw.cpp:148-164: the force factor is applied with the opposite sign */
        double f = p->sa1 + p->sa2 * r + p->sa3 * r * r;
        *fr = -f;
        *half_e = 0.5 * (p->sa0 + f * r);
    } else {
        /* sw.cpp:166-189 */
        double ira = 1.0 / (r - k->rc);
        double rp = pow(r, -p->p);
        double rq = pow(r, -p->q);
        double fex = exp(p->sigma * ira);
        *fr = (k->c1 * rp - k->c2 * rq + (k->c3 * rp - k->c4 * rq) * ira * ira * r) * fex / (r * r);
        *half_e = 0.5 * (k->c5 * rp - k->c6 * rq) * fex;
    }
}

int oc_sw(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j, const int* nbr_code,
          const oc_sw_param* p, double* f, double* e, double* vir) {
    sw_const k;
    sw_constants(p, &k);
    double rcsq = k.rc * k.rc;
    zero3(n, f, e, vir);
    for (int i = 0; i < n; i++) {
        for (int a = offsets[i]; a < offsets[i + 1]; a++) {
            int j = nbr_j[a];
            double s[3], d[3];
            shift_vec(box, nbr_code[a], s);
            double r2 = pair_dist2(x + 3 * i, x + 3 * j, s, d);
            if (!(r2 < rcsq)) continue;
            double r = sqrt(r2), fr, he;
            sw_two_body(p, &k, r, &fr, &he);
            f[3 * i + 0] += d[0] * fr;
            f[3 * i + 1] += d[1] * fr;
            f[3 * i + 2] += d[2] * fr;
            e[i] += he;
            vir[i] += d[0] * fr * d[0] + d[1] * fr * d[1] + d[2] * fr * d[2];
        }
    }
    /* three-body, sw.cpp:191-236 and :254-273: centre i, j before k in the
       list; vectors point from the centre to the neighbour. */
    for (int i = 0; i < n; i++) {
        for (int a = offsets[i]; a < offsets[i + 1]; a++) {
            double s1[3], d1[3];
            int j = nbr_j[a];
            shift_vec(box, nbr_code[a], s1);
            double rr1 = pair_dist2(x + 3 * i, x + 3 * j, s1, d1);
            if (!(rr1 < rcsq)) continue;
            /* d = x_neighbour - x_centre */
            double dx1 = -d1[0], dy1 = -d1[1], dz1 = -d1[2];
            for (int b = a + 1; b < offsets[i + 1]; b++) {
                double s2[3], d2[3];
                int kk = nbr_j[b];
                shift_vec(box, nbr_code[b], s2);
                double rr2 = pair_dist2(x + 3 * i, x + 3 * kk, s2, d2);
                if (!(rr2 < rcsq)) continue;
                double dx2 = -d2[0], dy2 = -d2[1], dz2 = -d2[2];
                double r1 = sqrt(rr1), r2 = sqrt(rr2);
                double ira0 = 1.0 / (r1 - k.rc), ira1 = 1.0 / (r2 - k.rc);
                double fira0 = k.c7 * ira0, fira1 = k.c7 * ira1;
                double ir1r2 = 1.0 / (r1 * r2);
                double fex = exp(fira0) * exp(fira1);
                double costheta = (dx1 * dx2 + dy1 * dy2 + dz1 * dz2) * ir1r2;
                double dcos = costheta - k.c10;
                double dccos = dcos * dcos;
                double ftheta = k.c9 * fex * dcos;
                double ft12 = ir1r2 * ftheta;
                double fpot = k.c8 * fex * dccos;
                double fcos = costheta * ftheta;
                double fr0 = fpot * fira0 * ira0 / r1, fr1 = fpot * fira1 * ira1 / r2;
                double ft0 = fcos / (r1 * r1), ft1 = fcos / (r2 * r2);
                double fx0 = dx1 * (fr0 + ft0) - dx2 * ft12, fx1 = dx2 * (fr1 + ft1) - dx1 * ft12;
                double fy0 = dy1 * (fr0 + ft0) - dy2 * ft12, fy1 = dy2 * (fr1 + ft1) - dy1 * ft12;
                double fz0 = dz1 * (fr0 + ft0) - dz2 * ft12, fz1 = dz2 * (fr1 + ft1) - dz1 * ft12;
                f[3 * i + 0] -= fx0 + fx1;
                f[3 * i + 1] -= fy0 + fy1;
                f[3 * i + 2] -= fz0 + fz1;
                f[3 * j + 0] += fx0;
                f[3 * j + 1] += fy0;
                f[3 * j + 2] += fz0;
                f[3 * kk + 0] += fx1;
                f[3 * kk + 1] += fy1;
                f[3 * kk + 2] += fz1;
                double third = fpot * (1.0 / 3.0);
                e[i] += third;
                e[j] += third;
                e[kk] += third;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------- Tersoff */

static double ters_fc(const oc_tersoff_param* p, double r, double* dfc) {
    if (r < p->R - p->D) {
        *dfc = 0.0;
        return 1.0;
    }
    if (r < p->R + p->D) {
        double arg = M_PI * (r - p->R) / (2.0 * p->D);
        *dfc = -M_PI / (4.0 * p->D) * cos(arg);
        return 0.5 - 0.5 * sin(arg);
    }
    *dfc = 0.0;
    return 0.0;
}

int oc_tersoff(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j,
               const int* nbr_code, const oc_tersoff_param* p, double* f, double* e, double* vir) {
    double rcut = p->R + p->D;
    double c2 = p->c * p->c, d2 = p->d * p->d, l3c = p->lambda3 * p->lambda3 * p->lambda3;
    zero3(n, f, e, vir);
    enum { MAXN = 256 };
    int nb[MAXN];
    double rv[MAXN][3], rr[MAXN];
    for (int i = 0; i < n; i++) {
        /* neighbours within the cutoff; rv = x_neighbour - x_i */
        int m = 0;
        for (int a = offsets[i]; a < offsets[i + 1]; a++) {
            double s[3], d[3];
            shift_vec(box, nbr_code[a], s);
            double r2 = pair_dist2(x + 3 * i, x + 3 * nbr_j[a], s, d);
            double r = sqrt(r2);
            if (!(r < rcut)) continue;
            if (m == MAXN) return -1;
            nb[m] = nbr_j[a];
            rv[m][0] = -d[0];
            rv[m][1] = -d[1];
            rv[m][2] = -d[2];
            rr[m] = r;
            m++;
        }
        for (int a = 0; a < m; a++) {
            int j = nb[a];
            double rij = rr[a], uij[3] = {rv[a][0] / rij, rv[a][1] / rij, rv[a][2] / rij};
            /* zeta and its gradient with respect to x_j and each x_k (x_i by sum) */
            double zeta = 0.0;
            double gj[3] = {0, 0, 0};
            double gk[MAXN][3];
            for (int b = 0; b < m; b++) {
                gk[b][0] = gk[b][1] = gk[b][2] = 0.0;
                if (b == a) continue;
                double rik = rr[b], uik[3] = {rv[b][0] / rik, rv[b][1] / rik, rv[b][2] / rik};
                double cs = uij[0] * uik[0] + uij[1] * uik[1] + uij[2] * uik[2];
                double dfc, fc = ters_fc(p, rik, &dfc);
                double hc = p->h - cs;
                double den = d2 + hc * hc;
                double g = 1.0 + c2 / d2 - c2 / den;
                double dg = -2.0 * c2 * hc / (den * den);
                double dr = rij - rik;
                double ex = exp(l3c * dr * dr * dr);
                double dex = 3.0 * l3c * dr * dr * ex; /* d ex / d rij = - d ex / d rik */
                zeta += fc * g * ex;
                for (int q = 0; q < 3; q++) {
                    double dcos_dj = (uik[q] - cs * uij[q]) / rij;
                    double dcos_dk = (uij[q] - cs * uik[q]) / rik;
                    gj[q] += fc * dg * ex * dcos_dj + fc * g * dex * uij[q];
                    gk[b][q] += dfc * g * ex * uik[q] + fc * dg * ex * dcos_dk - fc * g * dex * uik[q];
                }
            }
            double dfc_ij, fc_ij = ters_fc(p, rij, &dfc_ij);
            double fr = p->A * exp(-p->lambda1 * rij), fa = p->B * exp(-p->lambda2 * rij);
            double bn = pow(p->beta * zeta, p->n);
            double bij = pow(1.0 + bn, -1.0 / (2.0 * p->n));
            double dbdz = 0.0;
            if (zeta > 0.0) dbdz = -0.5 * pow(1.0 + bn, -1.0 / (2.0 * p->n) - 1.0) * bn / zeta;
            double vij = fc_ij * (fr - bij * fa);
            double dv_dr = dfc_ij * (fr - bij * fa) + fc_ij * (-p->lambda1 * fr + bij * p->lambda2 * fa);
            double dv_dz = -fc_ij * fa * dbdz;
            /* E = 1/2 sum V_ij: gradient of 1/2 V_ij */
            double gxj[3], gxi[3] = {0, 0, 0};
            for (int q = 0; q < 3; q++) {
                gxj[q] = 0.5 * (dv_dr * uij[q] + dv_dz * gj[q]);
                gxi[q] -= gxj[q];
            }
            for (int b = 0; b < m; b++) {
                if (b == a) continue;
                for (int q = 0; q < 3; q++) {
                    double g = 0.5 * dv_dz * gk[b][q];
                    f[3 * nb[b] + q] -= g;
                    gxi[q] -= g;
                }
            }
            for (int q = 0; q < 3; q++) {
                f[3 * j + q] -= gxj[q];
                f[3 * i + q] -= gxi[q];
            }
            e[i] += 0.5 * vij;
            vir[i] += 0.5 * dv_dr * rij; /* radial part only */
        }
    }
    return 0;
}

/* ------------------------------------------------------------ integrator */

void oc_vv_kick_drift(int n, double* x, double* v, const double* f, const double* mass, double dt) {
    double half_dt = 0.5 * dt;
    for (int i = 0; i < n; i++) {
        /* integrator.cpp:236-241: v += half_dt*f/Mass, then x += dt*v */
        for (int q = 0; q < 3; q++) v[3 * i + q] += half_dt * f[3 * i + q] / mass[i];
        for (int q = 0; q < 3; q++) x[3 * i + q] += dt * (v[3 * i + q]);
    }
}

void oc_vv_kick(int n, double* v, const double* f, const double* mass, double dt) {
    double half_dt = 0.5 * dt;
    for (int i = 0; i < n; i++)
        for (int q = 0; q < 3; q++) v[3 * i + q] += half_dt * f[3 * i + q] / mass[i];
}

double oc_kinetic(int n, const double* v, const double* mass) {
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        double sq = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
        s += mass[i] * sq;
    }
    return 0.5 * s;
}

void oc_wrap(const oc_box* box, int n, double* x) {
    for (int d = 0; d < 3; d++) {
        if (!box->periodic[d]) continue;
        double L = box->hi[d] - box->lo[d];
        for (int i = 0; i < n; i++) {
            int u = (int)floor((x[3 * i + d] - box->lo[d]) / L);
            if (u < 0) x[3 * i + d] = x[3 * i + d] + L;
            else if (u >= 1) x[3 * i + d] = x[3 * i + d] + (-L);
        }
    }
}

double oc_berendsen_factor(double dt, double tau, double tset, double tnow) {
    if (tnow <= 0.0) return 1.0;
    return sqrt(1. + dt / tau * (tset / tnow - 1.));
}
