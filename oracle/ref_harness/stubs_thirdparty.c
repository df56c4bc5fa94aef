/*
 * Stand-ins for the third-party libraries the reference links but the
 * checked path never calls: PARDISO 5.0 (absent from the reference tree)
 * and HSL MC73 (Fortran, no compiler here).  Calling one is an error.
 */
#include <stdio.h>
#include <stdlib.h>

static void femref_unavailable(const char *what)
{
    fprintf(stderr, "%s is not available in the checker build\n", what);
    abort();
}
void pardisoinit(void *a, int *b, int *c, int *d, double *e, int *f)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; femref_unavailable("PARDISO"); }
void pardiso(void *a, int *b, int *c, int *d, int *e, int *f, double *g, int *h, int *i,
             int *j, int *k, int *l, int *m, double *n, double *o, int *p, double *q)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i;
  (void)j; (void)k; (void)l; (void)m; (void)n; (void)o; (void)p; (void)q;
  femref_unavailable("PARDISO"); }
void pardiso_chkmatrix(int *a, int *b, double *c, int *d, int *e, int *f)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; femref_unavailable("PARDISO"); }
void pardiso_chkvec(int *a, int *b, double *c, int *d)
{ (void)a; (void)b; (void)c; (void)d; femref_unavailable("PARDISO"); }
void pardiso_printstats(int *a, int *b, double *c, int *d, int *e, int *f, double *g, int *h)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; femref_unavailable("PARDISO"); }
void mc73_fiedler(int *n, int *lirn, int *irn, int *ip, int *list, double *fv, int *info, double *a)
{ (void)n; (void)lirn; (void)irn; (void)ip; (void)list; (void)fv; (void)info; (void)a;
  femref_unavailable("HSL MC73"); }
