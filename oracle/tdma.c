/*
 * ORACLE — test infrastructure only.  Plain-C restatement of the reference's
 * serial Thomas solver ``tdma`` (ionization/cy.pyx:9-50), used as the parity
 * checker and as the timed CPU baseline.  It is never linked into, or called
 * by, the product library.
 *
 * Conventions follow cy.pyx exactly:
 *   sub[i]   (i = 0..n-2) multiplies x[i]   in row i+1   (cy.pyx:19, data[0])
 *   diag[i]  (i = 0..n-1)                                 (cy.pyx:20, data[1])
 *   sup[i]   (i = 0..n-2) multiplies x[i+1] in row i      (cy.pyx:21, data[2,1:])
 * Forward elimination  cy.pyx:31-43, back substitution  cy.pyx:45-48.
 * No pivoting; a zero pivot yields inf/nan, as in the reference
 * (cdivision=True).
 *
 * ``oracle_tdma_batched`` applies the same recurrence to ``nsys`` independent
 * systems stored back to back (system s occupies [s*n, (s+1)*n)); ``sub`` and
 * ``sup`` then hold n-1 entries per system (stride n-1).
 */
#include <complex.h>
#include <stddef.h>
#include <stdlib.h>

typedef double _Complex cdouble;

static void thomas(ptrdiff_t n, const cdouble *sub, const cdouble *diag,
                   const cdouble *sup, const cdouble *d, cdouble *x,
                   cdouble *new_sup, cdouble *new_d) {
    if (n <= 0) return;
    if (n == 1) {
        x[0] = d[0] / diag[0];
        return;
    }
    new_sup[0] = sup[0] / diag[0];
    new_d[0] = d[0] / diag[0];
    for (ptrdiff_t i = 1; i < n - 1; ++i) {
        cdouble sub_i = sub[i - 1];
        cdouble denom = diag[i] - sub_i * new_sup[i - 1];
        new_sup[i] = sup[i] / denom;
        new_d[i] = (d[i] - sub_i * new_d[i - 1]) / denom;
    }
    new_d[n - 1] = (d[n - 1] - sub[n - 2] * new_d[n - 2]) /
                   (diag[n - 1] - sub[n - 2] * new_sup[n - 2]);
    x[n - 1] = new_d[n - 1];
    for (ptrdiff_t i = n - 2; i >= 0; --i) x[i] = new_d[i] - new_sup[i] * x[i + 1];
}

/* One system of length n (the cy.tdma call).  Returns 0, or -1 on bad size
 * or allocation failure. */
int oracle_tdma(ptrdiff_t n, const cdouble *sub, const cdouble *diag,
                const cdouble *sup, const cdouble *d, cdouble *x) {
    if (n < 0) return -1;
    cdouble *work = (cdouble *)malloc(sizeof(cdouble) * (size_t)(2 * (n > 0 ? n : 1)));
    if (!work) return -1;
    thomas(n, sub, diag, sup, d, x, work, work + n);
    free(work);
    return 0;
}

int oracle_tdma_batched(ptrdiff_t nsys, ptrdiff_t n, const cdouble *sub,
                        const cdouble *diag, const cdouble *sup,
                        const cdouble *d, cdouble *x) {
    if (nsys < 0 || n < 0) return -1;
    cdouble *work = (cdouble *)malloc(sizeof(cdouble) * (size_t)(2 * (n > 0 ? n : 1)));
    if (!work) return -1;
    ptrdiff_t off_stride = n > 0 ? n - 1 : 0;
    for (ptrdiff_t s = 0; s < nsys; ++s)
        thomas(n, sub + s * off_stride, diag + s * n, sup + s * off_stride,
               d + s * n, x + s * n, work, work + n);
    free(work);
    return 0;
}
