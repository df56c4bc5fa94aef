/*
 * CPU restatement of the time-integration schemes of
 * 00_CommonFiles/Time_Integration for one rank, shared by the Euler and the
 * transient-transport restatements (test infrastructure: the checker the
 * device time loops are compared with, never a product path).
 *
 *   OR_TIME_PREDICTOR  Predictor_Old.c:53-126; with a `predict` hook (the
 *                      bubble unknowns of the DD builds, updated by the
 *                      caller's correction) Predictor_New.c:67-159
 *   OR_TIME_BDF        Predictor_Old_BDF.c:44-150
 *   OR_TIME_TRBDF2     Predictor_New_TRBDF2.c:55-190 without the bubble
 *                      unknowns uB, aB (they feed only the DD builders)
 *
 * One correction (`correct`) is the Build at (u, a) with the given
 * Alpha_Build and DeltaT_Build, the preconditioner set-up on the residual
 * and the GMRES solve for Da.  The stop tests are Criteria.c:25-80; the
 * steady-state test reads the DeltaT in force when it runs (dtBDF2 for
 * TR-BDF2, Predictor_New_TRBDF2.c:127).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "femoracle.h"

static void axpy(int n, double a, const double *x, double *y)
{
    /* daxpy.c: y += a x (the unrolled loop rounds as the plain one) */
    for (int i = 0; i < n; i++) y[i] += a * x[i];
}

typedef struct {
    int neq, steps, corrections, gmres;
    const or_time_opts *to;
    or_correction_fn correct;
    void *ctx;
    double *Da, *diff;
} loop_state;

/* The multicorrection of every scheme: a += Da, u += coef Da until the
 * correction stop test (Criteria.c:25-41). */
static int multicorrect(loop_state *L, double alpha_b, double dt_b, double coef, double *u, double *a)
{
    int it = 0, stop;
    do {
        int gi = 0;
        it++;
        if (L->correct(L->ctx, alpha_b, dt_b, u, a, L->Da, &gi)) return -1;
        L->gmres += gi;
        axpy(L->neq, 1, L->Da, a);
        axpy(L->neq, coef, L->Da, u);
        double norm_a = sqrt(or_ddot(L->neq, a, a));
        double norm_Da = sqrt(or_ddot(L->neq, L->Da, L->Da));
        if (L->to->stop_by_norm) stop = norm_Da < L->to->correction_tol * norm_a || it >= L->to->max_corrections;
        else stop = it >= L->to->max_corrections;
    } while (!stop);
    L->corrections += it;
    return 0;
}

/* Criteria.c:44-80, plus the optional bound on the steps */
static int stop_time(loop_state *L, const double *u, const double *u_old, double t, double dt_now)
{
    int stop;
    if (L->to->steady_state) {
        for (int i = 0; i < L->neq; i++) L->diff[i] = u[i] - u_old[i];
        double nd = sqrt(or_ddot(L->neq, L->diff, L->diff)), nu = sqrt(or_ddot(L->neq, u, u));
        stop = L->to->time_tol * nu > nd || fabs(L->to->final_time - t) < dt_now;
    } else {
        stop = L->to->final_time - t < 1e-10;
    }
    if (L->to->max_steps > 0 && L->steps >= L->to->max_steps) stop = 1;
    return stop;
}

int or_time_integrate(int neq, double alpha, double dt, const or_time_opts *to, or_correction_fn correct,
                      void *ctx, double *u, double *a, or_time_stats *st)
{
    return or_time_integrate_ex(neq, alpha, dt, to, correct, NULL, ctx, u, a, st);
}

int or_time_integrate_ex(int neq, double alpha, double dt, const or_time_opts *to, or_correction_fn correct,
                         or_bubble_fn bubble, void *ctx, double *u, double *a, or_time_stats *st)
{
    size_t nb = sizeof(double) * ((size_t)neq + 1);
    double *u_old = calloc(1, nb), *u1 = calloc(1, nb), *u2 = calloc(1, nb);
    loop_state L = { neq, 0, 0, 0, to, correct, ctx, calloc(1, nb), calloc(1, nb) };
    double t = 0.0;
    int rc = 0, i;
    memset(a, 0, sizeof(double) * (size_t)neq);
    if (to->scheme == OR_TIME_PREDICTOR) {
        do {
            L.steps++;
            t += dt;
            memcpy(u_old, u, sizeof(double) * (size_t)neq);
            axpy(neq, (1.0 - alpha) * dt, a, u);                      /* prediction */
            memset(a, 0, sizeof(double) * (size_t)neq);
            if (bubble) bubble(ctx, OR_B_PREDICT, (1.0 - alpha) * dt, 0.0, u);  /* Predictor_New.c:82-83 */
            if ((rc = multicorrect(&L, alpha, dt, alpha * dt, u, a))) break;
        } while (!stop_time(&L, u, u_old, t, dt));
    } else if (to->scheme == OR_TIME_BDF) {
        const double four_thirds = 4.0 / 3.0, two_thirds = 2.0 / 3.0, one_third = 1.0 / 3.0;
        /* BDF1 start (:49-90): no prediction; the update uses the caller's
         * alpha while the Build keeps Alpha_Build = alpha throughout */
        L.steps++;
        t += dt;
        memcpy(u_old, u, sizeof(double) * (size_t)neq);
        memcpy(u1, u, sizeof(double) * (size_t)neq);
        memset(a, 0, sizeof(double) * (size_t)neq);
        rc = multicorrect(&L, alpha, dt, alpha * dt, u, a);
        memcpy(u2, u, sizeof(double) * (size_t)neq);
        /* BDF2 steps (:95-145); u_old keeps the initial state */
        if (!rc) do {
            L.steps++;
            t += dt;
            for (i = 0; i < neq; i++) {
                u[i] = four_thirds * u2[i] - one_third * u1[i];
                a[i] = 0.0;
            }
            if ((rc = multicorrect(&L, alpha, dt, two_thirds * dt, u, a))) break;
            memcpy(u1, u2, sizeof(double) * (size_t)neq);
            memcpy(u2, u, sizeof(double) * (size_t)neq);
        } while (!stop_time(&L, u, u_old, t, dt));
    } else if (to->scheme == OR_TIME_TRBDF2) {
        const double lambda = 2.0 - sqrt(2.0);
        const double A = 1.0 / (lambda * (2.0 - lambda));
        const double B = (1.0 - lambda) * (1.0 - lambda) / (lambda * (2.0 - lambda));
        const double dtTR = lambda * dt, dtBDF2 = (1.0 - lambda) * dt;
        const double aTR = 0.5, aBDF2 = 1.0 / (2.0 - lambda);
        if (bubble) bubble(ctx, OR_B_TRBDF2_START, 0.0, 0.0, u);     /* Predictor_New_TRBDF2.c:63 */
        memcpy(u_old, u, sizeof(double) * (size_t)neq);
        do {
            L.steps++;
            t += dtTR;                                                /* TR stage */
            axpy(neq, aTR * dtTR, a, u);
            memset(a, 0, sizeof(double) * (size_t)neq);
            if (bubble) bubble(ctx, OR_B_PREDICT, aTR * dtTR, 0.0, u);
            if ((rc = multicorrect(&L, aTR, dtTR, aTR * dtTR, u, a))) break;
            t += dtBDF2;                                              /* BDF2 stage */
            for (i = 0; i < neq; i++) {
                u[i] = A * u[i] - B * u_old[i];
                a[i] = 0.0;
            }
            if (bubble) bubble(ctx, OR_B_TRBDF2_COMBINE, A, B, u);
            if ((rc = multicorrect(&L, aBDF2, dtBDF2, aBDF2 * dtBDF2, u, a))) break;
            memcpy(u_old, u, sizeof(double) * (size_t)neq);
            if (bubble) bubble(ctx, OR_B_TRBDF2_SAVE, 0.0, 0.0, u);
        } while (!stop_time(&L, u, u_old, t, dtBDF2));
    } else if (to->scheme == OR_TIME_NEW_BDF) {
        /* Predictor_New_BDF.c:54-184: a BDF1 step with Alpha_Build = 1
         * (u += dt Da), then BDF2 steps with Alpha_Build = 2/3; each step
         * keeps u_old = u before its prediction for the steady-state test */
        const double four_thirds = 4.0 / 3.0, two_thirds = 2.0 / 3.0, one_third = 1.0 / 3.0;
        L.steps++;
        t += dt;
        memcpy(u1, u, sizeof(double) * (size_t)neq);
        memset(a, 0, sizeof(double) * (size_t)neq);
        if (bubble) bubble(ctx, OR_B_BDF_START, 0.0, 0.0, u);
        rc = multicorrect(&L, 1.0, dt, dt, u, a);
        memcpy(u2, u, sizeof(double) * (size_t)neq);
        if (bubble) bubble(ctx, OR_B_BDF_SAVE2, 0.0, 0.0, u);
        if (!rc) do {
            L.steps++;
            t += dt;
            memcpy(u_old, u, sizeof(double) * (size_t)neq);
            for (i = 0; i < neq; i++) {
                u[i] = four_thirds * u2[i] - one_third * u1[i];
                a[i] = 0.0;
            }
            if (bubble) bubble(ctx, OR_B_BDF_COMBINE, four_thirds, one_third, u);
            if ((rc = multicorrect(&L, 2.0 / 3.0, dt, two_thirds * dt, u, a))) break;
            memcpy(u1, u2, sizeof(double) * (size_t)neq);
            memcpy(u2, u, sizeof(double) * (size_t)neq);
            if (bubble) bubble(ctx, OR_B_BDF_SHIFT, 0.0, 0.0, u);
        } while (!stop_time(&L, u, u_old, t, dt));
    } else {
        rc = -1;
    }
    if (st) { st->steps = L.steps; st->corrections = L.corrections; st->gmres_iterations = L.gmres; st->t = t; }
    free(u_old); free(u1); free(u2); free(L.Da); free(L.diff);
    return rc ? -1 : L.steps;
}
