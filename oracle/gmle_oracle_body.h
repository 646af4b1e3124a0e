/*
 * Precision-generic body of the CPU oracle. TEST INFRASTRUCTURE ONLY: the
 * product library never links or calls this code.
 *
 * Included twice by gmle_oracle.c: once with R = float (an op-for-op
 * restatement of the reference's FP32 CPU path, the parity target) and once
 * with R = double (the FP64 oracle of the same iteration, used to state each
 * result's error).  Every function cites the reference file:line it restates;
 * the evaluation order of each expression follows the Julia source so that
 * FP32 rounding matches (Julia does not contract a*b+c into an FMA, and the
 * oracle is compiled with -ffp-contract=off).
 *
 * Macros supplied by the includer:
 *   R        element type (float | double)
 *   FN(x)    name mangler (x##_f32 | x##_f64)
 *   ERF EXP LOG SQRT          libm functions of type R
 *   POW4(x) POW5(x) POW15(x)  Julia's x^4, x^5, x^1.5f0 for type R
 */

/* ---- Julia scalar semantics ------------------------------------------------ */

/* Base.max for IEEE floats: NaN-propagating, +0 > -0. */
static inline R FN(jl_max)(R x, R y)
{
    if (isnan(x) || isnan(y)) return x + y;
    R diff = x - y;
    return signbit(diff) ? y : x;
}

/* Base.min for IEEE floats. */
static inline R FN(jl_min)(R x, R y)
{
    if (isnan(x) || isnan(y)) return x + y;
    R diff = x - y;
    return signbit(diff) ? x : y;
}

/* Base.clamp: ifelse(x > hi, hi, ifelse(x < lo, lo, x)); NaN passes through. */
static inline R FN(jl_clamp)(R x, R lo, R hi)
{
    return x > hi ? hi : (x < lo ? lo : x);
}

/* sqrt(two * one(T) * pi) as Julia evaluates it in type R. */
static inline R FN(sqrt2pi)(void)
{
    return SQRT((R)2 * (R)3.14159265358979323846);
}

/* ---- GaussLib primitives: src/gausslib/baselibrary.jl ----------------------- */

/* integral_gaussian_1d, src/gausslib/baselibrary.jl:8-14 */
static inline R FN(integral_gaussian_1d)(int i, R pos, R sigma)
{
    const R half = (R)0.5;
    R norm = half / (sigma * sigma);
    R s = SQRT(norm);
    return half * (ERF(((R)i - pos + half) * s) - ERF(((R)i - pos - half) * s));
}

/* derivative_integral_gaussian_1d, src/gausslib/baselibrary.jl:21-33 */
static inline void FN(deriv_1d)(int ii, R x, R sigma, R N, R psf_other, R *dudt, R *d2)
{
    const R half = (R)0.5;
    R ta = ((R)ii + half - x) / sigma;
    R tb = ((R)ii - half - x) / sigma;
    R fa = EXP(-half * (ta * ta));
    R fb = EXP(-half * (tb * tb));
    R constant = -N / FN(sqrt2pi)() / sigma;
    *dudt = constant * (fa - fb) * psf_other;
    *d2 = constant / (sigma * sigma) *
          (((R)ii + half - x) * fa - ((R)ii - half - x) * fb) * psf_other;
}

/* derivative_integral_gaussian_1d_sigma, src/gausslib/baselibrary.jl:40-52 */
static inline void FN(deriv_1d_sigma)(int i, R x, R sx, R N, R psf_other, R *dudt, R *d2)
{
    const R half = (R)0.5;
    R ta = ((R)i + half - x) / sx;
    R tb = ((R)i - half - x) / sx;
    R ax = EXP(-half * (ta * ta));
    R bx = EXP(-half * (tb * tb));
    R ua = (R)i - x + half;
    R ub = (R)i - x - half;
    R c = FN(sqrt2pi)();
    R du = -N / c / sx / sx * (ax * ua - bx * ub) * psf_other;
    *dudt = du;
    *d2 = -(R)2 / sx * du -
          N / c / POW5(sx) * (ax * (ua * ua * ua) - bx * (ub * ub * ub)) * psf_other;
}

/* ---- per-pixel model and derivatives: src/psf_derivatives.jl --------------- */

/*
 * Fills model value, dudt[P] and the diagonal d2[P] at pixel (i = row, j = col)
 * for the parameter vector th.  psf[] holds the model constants in pixel units
 * (XYNB: psf[0] = sigma; astigmatic: sx0, sy0, Ax, Ay, Bx, By, gamma, d).
 */
static void FN(pixel_derivatives)(int model, int i, int j, const R *th, const R *psf,
                                  R *mu, R *dudt, R *d2)
{
    if (model == 0) { /* GaussianXYNB, src/psf_derivatives.jl:6-37 */
        R x = th[0], y = th[1], N = th[2], bg = th[3], s = psf[0];
        R px = FN(integral_gaussian_1d)(j, x, s);
        R py = FN(integral_gaussian_1d)(i, y, s);
        FN(deriv_1d)(j, x, s, N, py, &dudt[0], &d2[0]);
        FN(deriv_1d)(i, y, s, N, px, &dudt[1], &d2[1]);
        *mu = bg + N * px * py;
        dudt[2] = px * py; dudt[3] = (R)1;
        d2[2] = 0; d2[3] = 0;
    } else if (model == 1) { /* GaussianXYNBS, src/psf_derivatives.jl:40-73 */
        R x = th[0], y = th[1], N = th[2], bg = th[3], s = th[4];
        R px = FN(integral_gaussian_1d)(j, x, s);
        R py = FN(integral_gaussian_1d)(i, y, s);
        FN(deriv_1d)(j, x, s, N, py, &dudt[0], &d2[0]);
        FN(deriv_1d)(i, y, s, N, px, &dudt[1], &d2[1]);
        /* derivative_integral_gaussian_2d_sigma, baselibrary.jl:61-67 */
        R dsx, ddsx, dsy, ddsy;
        FN(deriv_1d_sigma)(j, x, s, N, py, &dsx, &ddsx);
        FN(deriv_1d_sigma)(i, y, s, N, px, &dsy, &ddsy);
        *mu = bg + N * px * py;
        dudt[2] = px * py; dudt[3] = (R)1; dudt[4] = dsx + dsy;
        d2[2] = 0; d2[3] = 0; d2[4] = ddsx + ddsy;
    } else if (model == 2) { /* GaussianXYNBSXSY, src/psf_derivatives.jl:76-112 */
        R x = th[0], y = th[1], N = th[2], bg = th[3], sx = th[4], sy = th[5];
        R px = FN(integral_gaussian_1d)(j, x, sx);
        R py = FN(integral_gaussian_1d)(i, y, sy);
        FN(deriv_1d)(j, x, sx, N, py, &dudt[0], &d2[0]);
        FN(deriv_1d)(i, y, sy, N, px, &dudt[1], &d2[1]);
        FN(deriv_1d_sigma)(j, x, sx, N, py, &dudt[4], &d2[4]);
        FN(deriv_1d_sigma)(i, y, sy, N, px, &dudt[5], &d2[5]);
        *mu = bg + N * px * py;
        dudt[2] = px * py; dudt[3] = (R)1;
        d2[2] = 0; d2[3] = 0;
    } else { /* AstigmaticXYZNB, src/psf_derivatives.jl:115-187 */
        R x = th[0], y = th[1], z = th[2], N = th[3], bg = th[4];
        R sx0 = psf[0], sy0 = psf[1], Ax = psf[2], Ay = psf[3], Bx = psf[4], By = psf[5];
        R gam = psf[6], d = psf[7];
        R zdx = (z - gam) / d;
        R ax = (R)1 + zdx * zdx + Ax * (zdx * zdx * zdx) + Bx * POW4(zdx);
        R zdy = (z + gam) / d;
        R ay = (R)1 + zdy * zdy + Ay * (zdy * zdy * zdy) + By * POW4(zdy);
        R sx = sx0 * SQRT(ax);
        R sy = sy0 * SQRT(ay);
        R px = FN(integral_gaussian_1d)(j, x, sx);
        R py = FN(integral_gaussian_1d)(i, y, sy);
        R dux, d2x, duy, d2y, dsx, ddsx, dsy, ddsy;
        FN(deriv_1d)(j, x, sx, N, py, &dux, &d2x);
        FN(deriv_1d)(i, y, sy, N, px, &duy, &d2y);
        FN(deriv_1d_sigma)(j, x, sx, N, py, &dsx, &ddsx);
        FN(deriv_1d_sigma)(i, y, sy, N, px, &dsy, &ddsy);
        R dax = ((R)2 * zdx + (R)3 * Ax * (zdx * zdx) + (R)4 * Bx * (zdx * zdx * zdx)) / d;
        R day = ((R)2 * zdy + (R)3 * Ay * (zdy * zdy) + (R)4 * By * (zdy * zdy * zdy)) / d;
        R dsx_dz = (sx0 / ((R)2 * SQRT(ax))) * dax;
        R dsy_dz = (sy0 / ((R)2 * SQRT(ay))) * day;
        R du_z = dsx * dsx_dz + dsy * dsy_dz;
        R d2ax = ((R)2 + (R)6 * Ax * zdx + (R)12 * Bx * (zdx * zdx)) / (d * d);
        R d2ay = ((R)2 + (R)6 * Ay * zdy + (R)12 * By * (zdy * zdy)) / (d * d);
        R d2sx = -(sx0 / ((R)4 * POW15(ax))) * (dax * dax) + (sx0 / ((R)2 * SQRT(ax))) * d2ax;
        R d2sy = -(sy0 / ((R)4 * POW15(ay))) * (day * day) + (sy0 / ((R)2 * SQRT(ay))) * d2ay;
        R d2z = ddsx * (dsx_dz * dsx_dz) + dsx * d2sx + ddsy * (dsy_dz * dsy_dz) + dsy * d2sy;
        *mu = bg + N * px * py;
        dudt[0] = dux; dudt[1] = duy; dudt[2] = du_z; dudt[3] = px * py; dudt[4] = (R)1;
        d2[0] = d2x; d2[1] = d2y; d2[2] = d2z; d2[3] = 0; d2[4] = 0;
    }
}

/* ---- camera likelihood terms: src/camera_models.jl -------------------------- */

/* compute_likelihood_terms (Poisson) src/camera_models.jl:19-34 and
 * (sCMOS variance map) :36-42 */
static inline void FN(likelihood_terms)(int scmos, R data, R mu, R var, R *cf, R *df)
{
    if (!scmos) {
        if (mu > (R)0.01f) {
            R c = data / mu - (R)1;
            R d = data / (mu * mu);
            *cf = FN(jl_min)(c, (R)1e4f);
            *df = FN(jl_min)(d, (R)1e4f);
        } else {
            *cf = 0; *df = 0;
        }
    } else {
        R tv = mu + var;
        *cf = (data - mu) / tv;
        *df = (R)1 / tv;
    }
}

/* compute_log_likelihood: Poisson src/camera_models.jl:60-71, sCMOS :73-85 */
static inline R FN(log_likelihood_term)(int scmos, R data, R mu, R var)
{
    if (!scmos) {
        if (mu > 0 && data > 0) return data * LOG(mu) - mu - (data * LOG(data) - data);
        if (mu > 0 && data == 0) return -mu;
        return 0;
    }
    R tv = mu + var;
    if (tv > 0) {
        R r = data - mu;
        return -(R)0.5 * ((r * r) / tv);
    }
    return 0;
}

/* ---- initialisation: src/unified_kernel.jl:158-255 -------------------------- */

static void FN(initialize)(int model, int box, const R *roi, const R *psf, R *th)
{
    /* simple_initialize_common, src/unified_kernel.jl:158-192 */
    R edge_sum = 0;
    int edge_count = 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++)
            if (i == 1 || i == box || j == 1 || j == box) {
                edge_sum += roi[(i - 1) + box * (j - 1)];
                edge_count++;
            }
    R bg = edge_sum / (R)edge_count;
    R total = 0, xw = 0, yw = 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++) {
            R sig = FN(jl_max)((R)0, roi[(i - 1) + box * (j - 1)] - bg);
            total += sig;
            xw += sig * (R)j;
            yw += sig * (R)i;
        }
    R center = (R)((box + 1) / 2.0);
    R x = total > (R)10 ? xw / total : center;
    R y = total > (R)10 ? yw / total : center;
    x = FN(jl_clamp)(x, (R)1.5, (R)(box - 0.5));
    y = FN(jl_clamp)(y, (R)1.5, (R)(box - 0.5));
    R photons = FN(jl_max)(total, (R)100);

    if (model == 0) { th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; return; }
    if (model == 1) { th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; th[4] = (R)1.3f; return; }
    if (model == 2) {
        th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; th[4] = (R)1.3f; th[5] = (R)1.3f;
        return;
    }
    /* astigmatic z from second moments, src/unified_kernel.jl:210-255 */
    R tot2 = 0, mxx = 0, myy = 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++) {
            R sig = FN(jl_max)((R)0, roi[(i - 1) + box * (j - 1)] - bg);
            tot2 += sig;
            R dx = (R)j - x, dy = (R)i - y;
            mxx += sig * dx * dx;
            myy += sig * dy * dy;
        }
    R z;
    if (tot2 > (R)10) {
        R sxe = SQRT(FN(jl_max)((R)0.5, mxx / tot2));
        R sye = SQRT(FN(jl_max)((R)0.5, myy / tot2));
        R rx = sxe / psf[0], ry = sye / psf[1];
        R dalpha = rx * rx - ry * ry;
        z = -dalpha * (psf[7] * psf[7]) / ((R)4 * psf[6]);
        z = FN(jl_clamp)(z, (R)-600, (R)600);
    } else {
        z = 0;
    }
    th[0] = x; th[1] = y; th[2] = z; th[3] = photons; th[4] = bg;
}

/* ---- small dense linear algebra: src/unified_kernel.jl:7-137 ---------------- */

/* static_cholesky_decomposition!, src/unified_kernel.jl:7-29 (A column-major NxN) */
static int FN(cholesky)(R *A, int n)
{
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) {
            R s = A[i + n * j];
            for (int k = 0; k < j; k++) s -= A[i + n * k] * A[j + n * k];
            if (i == j) {
                if (s <= 0) return 0;
                A[i + n * i] = SQRT(s);
            } else {
                A[i + n * j] = s / A[j + n * j];
            }
        }
    return 1;
}

/* static_cholesky_inverse!, src/unified_kernel.jl:32-60: diagonal of (L L^T)^-1 */
static void FN(cholesky_inverse_diag)(const R *L, int n, R *diag)
{
    R Li[36];
    for (int j = 0; j < n; j++) {
        Li[j + n * j] = (R)1 / L[j + n * j];
        for (int i = j + 1; i < n; i++) {
            R s = 0;
            for (int k = j; k < i; k++) s += L[i + n * k] * Li[k + n * j];
            Li[i + n * j] = -s / L[i + n * i];
        }
    }
    for (int i = 0; i < n; i++) {
        R s = 0;
        for (int k = i; k < n; k++) s += Li[k + n * i] * Li[k + n * i];
        diag[i] = s;
    }
}

/* maximum(abs, A) with Julia's NaN-propagating max */
static R FN(max_abs)(const R *A, int count)
{
    R m = FABS(A[0]);
    for (int t = 1; t < count; t++) m = FN(jl_max)(m, FABS(A[t]));
    return m;
}

/* static_lu_decomposition! + static_matrix_inverse!, src/unified_kernel.jl:64-137.
 * Returns 0 when a pivot falls below 1e-10 * max|A|; fills the inverse's diagonal. */
static int FN(lu_inverse_diag)(const R *Ain, int n, R *diag)
{
    R A[36];
    for (int t = 0; t < n * n; t++) A[t] = Ain[t];
    R tol = (R)1e-10f * FN(max_abs)(A, n * n);
    for (int k = 0; k < n; k++) {
        if (FABS(A[k + n * k]) < tol) return 0;
        for (int i = k + 1; i < n; i++) {
            A[i + n * k] /= A[k + n * k];
            for (int j = k + 1; j < n; j++) A[i + n * j] -= A[i + n * k] * A[k + n * j];
        }
    }
    for (int col = 0; col < n; col++) {
        R x[6];
        for (int i = 0; i < n; i++) {
            x[i] = (i == col) ? (R)1 : (R)0;
            for (int j = 0; j < i; j++) x[i] -= A[i + n * j] * x[j];
        }
        for (int i = n - 1; i >= 0; i--) {
            for (int j = i + 1; j < n; j++) x[i] -= A[i + n * j] * x[j];
            x[i] /= A[i + n * i];
        }
        diag[col] = x[col];
    }
    return 1;
}

/*
 * CRLB from a Fisher matrix, src/unified_kernel.jl:399-431: 1e-10*max|F| on the
 * diagonal, Cholesky inverse, LU fallback, else Inf.  Returns the flag bits.
 */
static int FN(crlb_from_fisher)(R *F, int n, R *crlb)
{
    R reg = (R)1e-10f * FN(max_abs)(F, n * n);
    for (int k = 0; k < n; k++) F[k + n * k] += reg;
    R Lc[36], diag[6];
    for (int t = 0; t < n * n; t++) Lc[t] = F[t];
    int flags;
    if (FN(cholesky)(Lc, n)) {
        FN(cholesky_inverse_diag)(Lc, n, diag);
        for (int k = 0; k < n; k++) crlb[k] = SQRT(FN(jl_max)((R)0, diag[k]));
        flags = ORACLE_FLAG_CHOLESKY;
    } else if (FN(lu_inverse_diag)(F, n, diag)) {
        for (int k = 0; k < n; k++) crlb[k] = SQRT(FN(jl_max)((R)0, diag[k]));
        flags = ORACLE_FLAG_LU;
    } else {
        for (int k = 0; k < n; k++) crlb[k] = (R)INFINITY;
        flags = ORACLE_FLAG_SINGULAR;
    }
    if (isfinite(crlb[0])) flags |= ORACLE_FLAG_CONVERGED;
    return flags;
}

/* ---- the per-ROI fit: unified_gaussian_mle_kernel!, src/unified_kernel.jl:285-434 */

/* sCMOS preprocessing, src/camera_models.jl:110-113 (to_electrons) and the
 * camera-coordinate map lookup of src/unified_kernel.jl:277-282: the ROI's
 * pixels in e- and its variance tile. */
static void FN(stage_roi)(const oracle_desc *d, const float *roi_in, int32_t xc, int32_t yc,
                          const float *var, const float *gain, const float *offset, int32_t ny,
                          R *roi, R *vroi)
{
    const int box = d->box;
    const int scmos = d->camera != 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++) {
            int p = (i - 1) + box * (j - 1);
            R v = (R)roi_in[p];
            R mv = 0;
            if (scmos) {
                int64_t m = (int64_t)(yc + i - 1 - 1) + (int64_t)ny * (int64_t)(xc + j - 1 - 1);
                mv = (R)var[m];
                if (d->camera == 2) v = (v - (R)offset[m]) * (R)gain[m];
            }
            roi[p] = v;
            vroi[p] = mv;
        }
}

/* final pass: LLR + Fisher + CRLB at theta, src/unified_kernel.jl:354-431 */
static int FN(final_pass)(const oracle_desc *d, const R *roi, const R *vroi, const R *th,
                          const R *psf, R *out_crlb, R *out_llr)
{
    const int box = d->box, P = oracle_nparams(d->model);
    const int scmos = d->camera != 0;
    R llr = 0, F[36];
    for (int t = 0; t < P * P; t++) F[t] = 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++) {
            int p = (i - 1) + box * (j - 1);
            R mu, du[6], d2[6];
            FN(pixel_derivatives)(d->model, i, j, th, psf, &mu, du, d2);
            llr += FN(log_likelihood_term)(scmos, roi[p], mu, vroi[p]);
            if (mu > 0) {
                R v = scmos ? mu + vroi[p] : mu;
                for (int k = 0; k < P; k++)
                    for (int l = k; l < P; l++) {
                        R f = du[k] * du[l] / v;
                        F[k + P * l] += f;
                        if (k != l) F[l + P * k] += f;
                    }
            }
        }
    *out_llr = llr;
    return FN(crlb_from_fisher)(F, P, out_crlb);
}

/* The final pass alone at a given theta (the fitted parameters of another
 * implementation), for the error of its Fisher accumulation and inversion. */
static void FN(final_at)(const oracle_desc *d, const float *roi_in, int32_t xc, int32_t yc,
                         const float *var, const float *gain, const float *offset, int32_t ny,
                         const double *theta, R *out_crlb, R *out_llr, uint8_t *out_flags)
{
    const int P = oracle_nparams(d->model);
    R roi[ORACLE_MAX_BOX * ORACLE_MAX_BOX], vroi[ORACLE_MAX_BOX * ORACLE_MAX_BOX], psf[8], th[6];
    for (int t = 0; t < 8; t++) psf[t] = (R)d->psf[t];
    for (int k = 0; k < P; k++) th[k] = (R)theta[k];
    FN(stage_roi)(d, roi_in, xc, yc, var, gain, offset, ny, roi, vroi);
    *out_flags = (uint8_t)FN(final_pass)(d, roi, vroi, th, psf, out_crlb, out_llr);
}

static void FN(fit_one)(const oracle_desc *d, const float *roi_in, int32_t xc, int32_t yc,
                        const float *var, const float *gain, const float *offset, int32_t ny,
                        R *out_params, R *out_crlb, R *out_llr, uint8_t *out_flags)
{
    const int box = d->box, P = oracle_nparams(d->model);
    const int scmos = d->camera != 0;
    R roi[ORACLE_MAX_BOX * ORACLE_MAX_BOX], vroi[ORACLE_MAX_BOX * ORACLE_MAX_BOX];
    R psf[8], lo[6], hi[6], ms[6];
    for (int t = 0; t < 8; t++) psf[t] = (R)d->psf[t];
    for (int k = 0; k < P; k++) { lo[k] = d->lower[k]; hi[k] = d->upper[k]; ms[k] = d->max_step[k]; }
    FN(stage_roi)(d, roi_in, xc, yc, var, gain, offset, ny, roi, vroi);

    R th[6];
    FN(initialize)(d->model, box, roi, psf, th);

    if (d->method == 1) {
        /* the library's full-Hessian option (no reference counterpart): Fisher
         * scoring with Levenberg-Marquardt damping.  Each pass at a candidate
         * gives L, the gradient g_k = sum du_k cf and F_kl = sum du_k du_l / v
         * (mu > 0).  A candidate at least as likely as the best (to 1e-5 |L|)
         * is accepted (its g and F kept, lambda / 10); a worse one is rejected
         * (lambda x 10).  The next step solves (F + lambda diag F) s = g at the best
         * point by Cholesky (the diagonal step if that fails), clamped like the
         * reference's steps. */
        R thb[6], stp[6] = {0}, Lb = (R)-INFINITY, lam = (R)1e-3f, gb[6] = {0}, Fb[36];
        for (int k = 0; k < P; k++) thb[k] = th[k];
        for (int t = 0; t < P * P; t++) Fb[t] = 0;
        for (int it = 0; it < d->iterations; it++) {
            if (it > 0)
                for (int k = 0; k < P; k++)
                    th[k] = FN(jl_clamp)(thb[k] + FN(jl_clamp)(stp[k], -ms[k], ms[k]), lo[k], hi[k]);
            R L = 0, g[6] = {0}, Fm[36];
            for (int t = 0; t < P * P; t++) Fm[t] = 0;
            for (int j = 1; j <= box; j++)
                for (int i = 1; i <= box; i++) {
                    int p = (i - 1) + box * (j - 1);
                    R mu, du[6], d2[6], cf, df;
                    FN(pixel_derivatives)(d->model, i, j, th, psf, &mu, du, d2);
                    FN(likelihood_terms)(scmos, roi[p], mu, vroi[p], &cf, &df);
                    L += FN(log_likelihood_term)(scmos, roi[p], mu, vroi[p]);
                    for (int k = 0; k < P; k++) g[k] += du[k] * cf;
                    if (mu > 0) {
                        R v = scmos ? mu + vroi[p] : mu;
                        for (int k = 0; k < P; k++)
                            for (int l = k; l < P; l++) Fm[k + P * l] += du[k] * du[l] / v;
                    }
                }
            if (it == 0 || L >= Lb - (R)1e-5f * FABS(Lb)) {
                for (int k = 0; k < P; k++) { thb[k] = th[k]; gb[k] = g[k]; }
                for (int t = 0; t < P * P; t++) Fb[t] = Fm[t];
                Lb = L;
                lam = FN(jl_max)(lam * (R)0.1f, (R)1e-7f);
            } else {
                lam = FN(jl_min)(lam * (R)10, (R)1e7f);
            }
            R A[36], y[6];
            for (int k = 0; k < P; k++)
                for (int l = k; l < P; l++) A[l + P * k] = A[k + P * l] = Fb[k + P * l];
            for (int k = 0; k < P; k++) A[k + P * k] = Fb[k + P * k] + lam * Fb[k + P * k];
            if (FN(cholesky)(A, P)) {
                for (int i = 0; i < P; i++) {
                    R sm = gb[i];
                    for (int k = 0; k < i; k++) sm -= A[i + P * k] * y[k];
                    y[i] = sm / A[i + P * i];
                }
                for (int i = P - 1; i >= 0; i--) {
                    R sm = y[i];
                    for (int k = i + 1; k < P; k++) sm -= A[k + P * i] * stp[k];
                    stp[i] = sm / A[i + P * i];
                }
            } else {
                for (int k = 0; k < P; k++)
                    stp[k] = Fb[k + P * k] > 0 ? gb[k] / Fb[k + P * k] : (R)0;
            }
        }
        for (int k = 0; k < P; k++) th[k] = thb[k];
    }

    for (int it = 0; d->method == 0 && it < d->iterations; it++) {
        R g[6] = {0}, h[6] = {0};
        for (int j = 1; j <= box; j++)
            for (int i = 1; i <= box; i++) {
                int p = (i - 1) + box * (j - 1);
                R mu, du[6], d2[6], cf, df;
                FN(pixel_derivatives)(d->model, i, j, th, psf, &mu, du, d2);
                FN(likelihood_terms)(scmos, roi[p], mu, vroi[p], &cf, &df);
                for (int k = 0; k < P; k++) {
                    g[k] += du[k] * cf;
                    h[k] += d2[k] * cf - du[k] * du[k] * df;
                }
            }
        /* scalar Newton step + apply_constraints!, src/unified_kernel.jl:337-350,
         * src/constraints.jl:49-53 */
        for (int k = 0; k < P; k++) {
            R delta = FABS(h[k]) > (R)1e-10f ? g[k] / h[k] : (R)0;
            R step = FN(jl_clamp)(delta, -ms[k], ms[k]);
            th[k] = FN(jl_clamp)(th[k] - step, lo[k], hi[k]);
        }
    }

    /* final pass: LLR + Fisher, src/unified_kernel.jl:354-397 */
    R llr, crlb[6];
    int flags = FN(final_pass)(d, roi, vroi, th, psf, crlb, &llr);
    for (int k = 0; k < P; k++) { out_params[k] = th[k]; out_crlb[k] = crlb[k]; }
    *out_llr = llr;
    *out_flags = (uint8_t)flags;
}

/* CRLB at a fixed parameter vector (Poisson camera): the Fisher pass of
 * src/unified_kernel.jl:359-431 without the Newton iterations. */
static int FN(crlb_at_theta)(int model, int box, const float *psf_in, const double *theta,
                             R *crlb)
{
    R psf[8], th[6], F[36];
    int P = oracle_nparams(model);
    for (int t = 0; t < 8; t++) psf[t] = (R)psf_in[t];
    for (int k = 0; k < P; k++) th[k] = (R)theta[k];
    for (int t = 0; t < P * P; t++) F[t] = 0;
    for (int j = 1; j <= box; j++)
        for (int i = 1; i <= box; i++) {
            R mu, du[6], d2[6];
            FN(pixel_derivatives)(model, i, j, th, psf, &mu, du, d2);
            if (mu > 0)
                for (int k = 0; k < P; k++)
                    for (int l = k; l < P; l++) {
                        R f = du[k] * du[l] / mu;
                        F[k + P * l] += f;
                        if (k != l) F[l + P * k] += f;
                    }
        }
    return FN(crlb_from_fisher)(F, P, crlb);
}
