/*
 * Seeded synthetic problem generators for the Krylov benchmarks and tests.
 *
 * The reference (flecsolve) ships no matrix generator for these workloads: its
 * solver tests read SuiteSparse MatrixMarket files
 * (flecsolve/solvers/test/cg.cc:63-69) and its examples assemble operators
 * matrix-free over FleCSI meshes (examples/poisson/poisson.hh:34-67,
 * flecsolve/physics/volume_diffusion/diffusion.hh:115-207). These generators
 * produce the same kinds of operators as assembled CSR:
 *
 *   - 5-point / 7-point finite-volume diffusion -div(c grad u) on an n^d grid
 *     of unit cells with Dirichlet u = 0 on the domain boundary.  Every face
 *     carries one coefficient c_f; an interior face couples its two cells with
 *     -c_f and adds c_f to both diagonals, a boundary face adds c_f to its
 *     cell's diagonal only.  With c_f = 1 everywhere in 2-D this is the
 *     classic 5-point Poisson matrix (diagonal 4, off-diagonals -1).
 *   - log-normal cell coefficients k = exp(sigma * N(0,1)) with harmonic face
 *     averaging 2 k_a k_b / (k_a + k_b); boundary faces get 2 k (half-cell
 *     distance to the Dirichlet face).
 *   - 3-D first-order upwind convection-diffusion with a discretely
 *     divergence-free (staggered curl of an edge vector potential) vortex.
 *
 * Everything here is plain IEEE double arithmetic (compile with
 * -ffp-contract=off): the RNG is splitmix64, the normal sampler is Marsaglia's
 * polar method, and exp/log are computed by the series below instead of libm,
 * so the same seed gives bit-identical matrices on x86-64 and aarch64.
 *
 * Row order is lexicographic r = (k*n + j)*n + i; within a row the columns are
 * ascending (-z, -y, -x, diag, +x, +y, +z neighbours).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define FSP_API __attribute__((visibility("default")))

/* ---------------------------------------------------------------- RNG --- */

/* splitmix64 (Steele, Lea, Flood: "Fast splittable pseudorandom number
 * generators", OOPSLA 2014). */
static inline uint64_t sm64(uint64_t *s) {
	uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

/* uniform in [0, 1) with 53 random bits */
static inline double u01(uint64_t *s) {
	return (double)(sm64(s) >> 11) * 0x1.0p-53;
}

/* log(x) for finite x > 0: reduce to m in [sqrt(1/2), sqrt(2)), then
 * log(m) = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716, odd series to s^23. */
static double fsp_log(double x) {
	int e;
	double m = frexp(x, &e);
	if (m < 0.70710678118654752440) {
		m *= 2.0;
		e -= 1;
	}
	double s = (m - 1.0) / (m + 1.0);
	double s2 = s * s;
	double t = 1.0 / 23.0;
	for (int k = 21; k >= 1; k -= 2)
		t = t * s2 + 1.0 / (double)k;
	return 2.0 * s * t + (double)e * 0.69314718055994530942;
}

/* exp(x) for |x| < 700: x = k ln2 + r with a two-part ln2 (Cody & Waite),
 * |r| <= ln2/2, Taylor polynomial to r^20/20! in Horner form. */
static double fsp_exp(double x) {
	const double ln2_hi = 6.93147180369123816490e-01; /* 32 leading bits */
	const double ln2_lo = 1.90821492927058770002e-10; /* ln2 - ln2_hi     */
	double kf = floor(x * 1.44269504088896340736 + 0.5);
	double r = (x - kf * ln2_hi) - kf * ln2_lo;
	double t = 1.0;
	for (int k = 20; k >= 1; --k)
		t = 1.0 + t * r / (double)k;
	return ldexp(t, (int)kf);
}

/* standard normal pairs by Marsaglia's polar method */
typedef struct {
	uint64_t s;
	int have;
	double spare;
} normal_stream;

static double nrm(normal_stream *g) {
	if (g->have) {
		g->have = 0;
		return g->spare;
	}
	double u, v, q;
	do {
		u = 2.0 * u01(&g->s) - 1.0;
		v = 2.0 * u01(&g->s) - 1.0;
		q = u * u + v * v;
	} while (!(q > 0.0 && q < 1.0));
	double f = sqrt(-2.0 * fsp_log(q) / q);
	g->spare = v * f;
	g->have = 1;
	return u * f;
}

FSP_API double fsp_exp_(double x) { return fsp_exp(x); }
FSP_API double fsp_log_(double x) { return fsp_log(x); }

/* out[i] = lo + (hi - lo) * U[0,1), i in [0, n), from splitmix64(seed) */
FSP_API void fsp_uniform(uint64_t seed, int64_t n, double lo, double hi,
                         double *out) {
	uint64_t s = seed;
	double w = hi - lo;
	for (int64_t i = 0; i < n; ++i)
		out[i] = lo + w * u01(&s);
}

/* out[i] = mu + sigma * N(0,1) */
FSP_API void fsp_normal(uint64_t seed, int64_t n, double mu, double sigma,
                        double *out) {
	normal_stream g = {seed, 0, 0.0};
	for (int64_t i = 0; i < n; ++i)
		out[i] = mu + sigma * nrm(&g);
}

/* n uniform integers in [lo, hi] (used for batched system sizes) */
FSP_API void fsp_randint(uint64_t seed, int64_t n, int64_t lo, int64_t hi,
                         int64_t *out) {
	uint64_t s = seed;
	uint64_t span = (uint64_t)(hi - lo + 1);
	for (int64_t i = 0; i < n; ++i)
		out[i] = lo + (int64_t)(sm64(&s) % span);
}

/* ------------------------------------------------------ grid helpers --- */

/* number of rows of an n^dim grid */
FSP_API int64_t fsp_grid_rows(int dim, int64_t n) {
	return dim == 2 ? n * n : n * n * n;
}

/* nonzeros of the 5-point (dim 2) / 7-point (dim 3) pattern */
FSP_API int64_t fsp_grid_nnz(int dim, int64_t n) {
	if (dim == 2)
		return 5 * n * n - 4 * n;
	return 7 * n * n * n - 6 * n * n;
}

/* number of face coefficients (boundary faces included) */
FSP_API int64_t fsp_grid_faces(int dim, int64_t n) {
	if (dim == 2)
		return 2 * n * (n + 1);
	return 3 * n * n * (n + 1);
}

/* Face layout.
 * dim 3: [cx | cy | cz]; cx[(k*n + j)*(n+1) + f] is the x-face between
 *   cells (f-1, j, k) and (f, j, k), f in [0, n] (f = 0 and f = n are
 *   boundary faces); cy[(k*(n+1) + f)*n + i]; cz[(f*n + j)*n + i].
 * dim 2: [cx | cy]; cx[j*(n+1) + f], cy[f*n + i]. */
static inline int64_t fx3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return (k * n + j) * (n + 1) + i;
}
static inline int64_t fy3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return n * n * (n + 1) + (k * (n + 1) + j) * n + i;
}
static inline int64_t fz3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return 2 * n * n * (n + 1) + (k * n + j) * n + i;
}
static inline int64_t fx2(int64_t n, int64_t i, int64_t j) {
	return j * (n + 1) + i;
}
static inline int64_t fy2(int64_t n, int64_t i, int64_t j) {
	return n * (n + 1) + j * n + i;
}

/* all faces = c */
FSP_API void fsp_faces_const(int dim, int64_t n, double c, double *faces) {
	int64_t nf = fsp_grid_faces(dim, n);
	for (int64_t f = 0; f < nf; ++f)
		faces[f] = c;
}

/* cell k = exp(mu + sigma N(0,1)) in row order; interior faces harmonic
 * 2 ka kb / (ka + kb); boundary faces 2 k.  If cells != NULL the cell field
 * is returned too. */
FSP_API void fsp_faces_lognormal(int dim, int64_t n, double mu, double sigma,
                                 uint64_t seed, double *faces, double *cells) {
	int64_t N = fsp_grid_rows(dim, n);
	double *k = cells ? cells : (double *)malloc((size_t)N * sizeof(double));
	normal_stream g = {seed, 0, 0.0};
	for (int64_t r = 0; r < N; ++r)
		k[r] = fsp_exp(mu + sigma * nrm(&g));
#define HARM(a, b) ((2.0 * (a) * (b)) / ((a) + (b)))
	if (dim == 2) {
		for (int64_t j = 0; j < n; ++j)
			for (int64_t f = 0; f <= n; ++f) {
				double c;
				if (f == 0)
					c = 2.0 * k[j * n];
				else if (f == n)
					c = 2.0 * k[j * n + n - 1];
				else
					c = HARM(k[j * n + f - 1], k[j * n + f]);
				faces[fx2(n, f, j)] = c;
			}
		for (int64_t f = 0; f <= n; ++f)
			for (int64_t i = 0; i < n; ++i) {
				double c;
				if (f == 0)
					c = 2.0 * k[i];
				else if (f == n)
					c = 2.0 * k[(n - 1) * n + i];
				else
					c = HARM(k[(f - 1) * n + i], k[f * n + i]);
				faces[fy2(n, i, f)] = c;
			}
	}
	else {
		for (int64_t kk = 0; kk < n; ++kk)
			for (int64_t j = 0; j < n; ++j)
				for (int64_t f = 0; f <= n; ++f) {
					int64_t base = (kk * n + j) * n;
					double c;
					if (f == 0)
						c = 2.0 * k[base];
					else if (f == n)
						c = 2.0 * k[base + n - 1];
					else
						c = HARM(k[base + f - 1], k[base + f]);
					faces[fx3(n, f, j, kk)] = c;
				}
		for (int64_t kk = 0; kk < n; ++kk)
			for (int64_t f = 0; f <= n; ++f)
				for (int64_t i = 0; i < n; ++i) {
					double c;
					if (f == 0)
						c = 2.0 * k[(kk * n) * n + i];
					else if (f == n)
						c = 2.0 * k[(kk * n + n - 1) * n + i];
					else
						c = HARM(k[(kk * n + f - 1) * n + i],
						         k[(kk * n + f) * n + i]);
					faces[fy3(n, i, f, kk)] = c;
				}
		for (int64_t f = 0; f <= n; ++f)
			for (int64_t j = 0; j < n; ++j)
				for (int64_t i = 0; i < n; ++i) {
					double c;
					if (f == 0)
						c = 2.0 * k[j * n + i];
					else if (f == n)
						c = 2.0 * k[((n - 1) * n + j) * n + i];
					else
						c = HARM(k[((f - 1) * n + j) * n + i],
						         k[(f * n + j) * n + i]);
					faces[fz3(n, i, j, f)] = c;
				}
	}
#undef HARM
	if (!cells)
		free(k);
}

/* Assemble the diffusion matrix from face coefficients (layout above).
 * rowptr has N+1 entries, col/val nnz = fsp_grid_nnz(dim, n) entries.
 * The diagonal is summed in the fixed face order -z, -y, -x, +x, +y, +z. */
FSP_API void fsp_assemble_diffusion(int dim, int64_t n, const double *faces,
                                    int64_t *rowptr, int32_t *col,
                                    double *val) {
	int64_t off = 0;
	rowptr[0] = 0;
	if (dim == 2) {
		for (int64_t j = 0; j < n; ++j)
			for (int64_t i = 0; i < n; ++i) {
				int64_t r = j * n + i;
				double cs = faces[fy2(n, i, j)], cn = faces[fy2(n, i, j + 1)];
				double cw = faces[fx2(n, i, j)], ce = faces[fx2(n, i + 1, j)];
				double d = 0.0;
				d += cs;
				d += cw;
				d += ce;
				d += cn;
				if (j > 0) { col[off] = (int32_t)(r - n); val[off++] = -cs; }
				if (i > 0) { col[off] = (int32_t)(r - 1); val[off++] = -cw; }
				col[off] = (int32_t)r;
				val[off++] = d;
				if (i + 1 < n) { col[off] = (int32_t)(r + 1); val[off++] = -ce; }
				if (j + 1 < n) { col[off] = (int32_t)(r + n); val[off++] = -cn; }
				rowptr[r + 1] = off;
			}
	}
	else {
		int64_t n2 = n * n;
		for (int64_t k = 0; k < n; ++k)
			for (int64_t j = 0; j < n; ++j)
				for (int64_t i = 0; i < n; ++i) {
					int64_t r = (k * n + j) * n + i;
					double cb = faces[fz3(n, i, j, k)], ct = faces[fz3(n, i, j, k + 1)];
					double cs = faces[fy3(n, i, j, k)], cn = faces[fy3(n, i, j + 1, k)];
					double cw = faces[fx3(n, i, j, k)], ce = faces[fx3(n, i + 1, j, k)];
					double d = 0.0;
					d += cb;
					d += cs;
					d += cw;
					d += ce;
					d += cn;
					d += ct;
					if (k > 0) { col[off] = (int32_t)(r - n2); val[off++] = -cb; }
					if (j > 0) { col[off] = (int32_t)(r - n); val[off++] = -cs; }
					if (i > 0) { col[off] = (int32_t)(r - 1); val[off++] = -cw; }
					col[off] = (int32_t)r;
					val[off++] = d;
					if (i + 1 < n) { col[off] = (int32_t)(r + 1); val[off++] = -ce; }
					if (j + 1 < n) { col[off] = (int32_t)(r + n); val[off++] = -cn; }
					if (k + 1 < n) { col[off] = (int32_t)(r + n2); val[off++] = -ct; }
					rowptr[r + 1] = off;
				}
	}
}

/* ------------------------------------------ convection-diffusion (3-D) --- */

/* Seeded vector potential on cell edges.  Each component is
 * B(x,y,z) * sum_m a_m * phi_m(x,y,z), B = 64 x(1-x) y(1-y) z(1-z), with
 * phi_m the 10 monomials of degree <= 1 and the products of pairs in the
 * centred coordinates, and amplitudes a_m ~ U[-1,1].  B vanishes on the
 * domain boundary, so the staggered curl has zero normal flux through it. */
#define NMODES 10
static double psi_eval(const double *a, double x, double y, double z) {
	double X = x - 0.5, Y = y - 0.5, Z = z - 0.5;
	double phi[NMODES] = {1.0, X, Y, Z, X * Y, Y * Z, Z * X,
	                      X * X - Y * Y, Y * Y - Z * Z, X * Y * Z * 8.0};
	double s = 0.0;
	for (int m = 0; m < NMODES; ++m)
		s += a[m] * phi[m];
	double B = 64.0 * x * (1.0 - x) * y * (1.0 - y) * z * (1.0 - z);
	return B * s;
}

/* Face velocities (outflow through the +x/+y/+z face of cell (i,j,k)) of the
 * staggered curl u = curl(psi); h = 1 in index space, psi in [0,1]^3 coords
 * scaled by n.  ux[fx3], uy[fy3], uz[fz3] use the face layout above. */
static void vortex_faces(int64_t n, uint64_t seed, double *u) {
	double a[3][NMODES];
	uint64_t s = seed;
	for (int c = 0; c < 3; ++c)
		for (int m = 0; m < NMODES; ++m)
			a[c][m] = 2.0 * u01(&s) - 1.0;
	double dn = (double)n;
	/* psi_x on edges (x cell centre, y and z on nodes): x = (i+0.5)/n,
	   y = jn/n, z = kn/n; psi_y on (x node, y centre, z node); psi_z on
	   (x node, y node, z centre).  Node coordinates are divided, not
	   multiplied by 1/n, so the last node is exactly 1 and B vanishes. */
#define PX(i, jn, kn) psi_eval(a[0], ((i) + 0.5) / dn, (jn) / dn, (kn) / dn)
#define PY(in, j, kn) psi_eval(a[1], (in) / dn, ((j) + 0.5) / dn, (kn) / dn)
#define PZ(in, jn, k) psi_eval(a[2], (in) / dn, (jn) / dn, ((k) + 0.5) / dn)
	/* ux at x-face (f, j, k) = d psi_z / dy - d psi_y / dz as differences of
	   edge values (the overall scale is normalised by the caller). */
	for (int64_t k = 0; k < n; ++k)
		for (int64_t j = 0; j < n; ++j)
			for (int64_t f = 0; f <= n; ++f)
				u[fx3(n, f, j, k)] = (PZ(f, j + 1, k) - PZ(f, j, k)) -
				                     (PY(f, j, k + 1) - PY(f, j, k));
	for (int64_t k = 0; k < n; ++k)
		for (int64_t f = 0; f <= n; ++f)
			for (int64_t i = 0; i < n; ++i)
				u[fy3(n, i, f, k)] = (PX(i, f, k + 1) - PX(i, f, k)) -
				                     (PZ(i + 1, f, k) - PZ(i, f, k));
	for (int64_t f = 0; f <= n; ++f)
		for (int64_t j = 0; j < n; ++j)
			for (int64_t i = 0; i < n; ++i)
				u[fz3(n, i, j, f)] = (PY(i + 1, j, f) - PY(i, j, f)) -
				                     (PX(i, j + 1, f) - PX(i, j, f));
#undef PX
#undef PY
#undef PZ
}

/* 3-D upwind convection-diffusion: unit diffusion (interior faces 1, boundary
 * faces 2), plus first-order upwind convection with the seeded vortex scaled
 * so that max_f |u_f| = pe_max (cell Peclet number |u| h / D with h = D = 1).
 * Row r: for each face with outflow velocity F (positive out of the cell):
 *   diag += c_f + max(F, 0);  neighbour coefficient = -c_f + min(F, 0).
 * If vel != NULL it receives the scaled face velocities (face layout). */
FSP_API void fsp_assemble_convdiff3d(int64_t n, double pe_max, uint64_t seed,
                                     int64_t *rowptr, int32_t *col, double *val,
                                     double *vel) {
	int64_t nf = fsp_grid_faces(3, n);
	double *u = vel ? vel : (double *)malloc((size_t)nf * sizeof(double));
	vortex_faces(n, seed, u);
	double umax = 0.0;
	for (int64_t f = 0; f < nf; ++f)
		umax = fmax(umax, fabs(u[f]));
	double sc = umax > 0.0 ? pe_max / umax : 0.0;
	for (int64_t f = 0; f < nf; ++f)
		u[f] *= sc;
	int64_t off = 0, n2 = n * n;
	rowptr[0] = 0;
	for (int64_t k = 0; k < n; ++k)
		for (int64_t j = 0; j < n; ++j)
			for (int64_t i = 0; i < n; ++i) {
				int64_t r = (k * n + j) * n + i;
				/* outflow velocities: -u on the lower faces, +u on the upper */
				double Fb = -u[fz3(n, i, j, k)], Ft = u[fz3(n, i, j, k + 1)];
				double Fs = -u[fy3(n, i, j, k)], Fn = u[fy3(n, i, j + 1, k)];
				double Fw = -u[fx3(n, i, j, k)], Fe = u[fx3(n, i + 1, j, k)];
				double cb = k > 0 ? 1.0 : 2.0, ct = k + 1 < n ? 1.0 : 2.0;
				double cs = j > 0 ? 1.0 : 2.0, cn = j + 1 < n ? 1.0 : 2.0;
				double cw = i > 0 ? 1.0 : 2.0, ce = i + 1 < n ? 1.0 : 2.0;
				double d = 0.0;
				d += cb + fmax(Fb, 0.0);
				d += cs + fmax(Fs, 0.0);
				d += cw + fmax(Fw, 0.0);
				d += ce + fmax(Fe, 0.0);
				d += cn + fmax(Fn, 0.0);
				d += ct + fmax(Ft, 0.0);
				if (k > 0) { col[off] = (int32_t)(r - n2); val[off++] = -cb + fmin(Fb, 0.0); }
				if (j > 0) { col[off] = (int32_t)(r - n); val[off++] = -cs + fmin(Fs, 0.0); }
				if (i > 0) { col[off] = (int32_t)(r - 1); val[off++] = -cw + fmin(Fw, 0.0); }
				col[off] = (int32_t)r;
				val[off++] = d;
				if (i + 1 < n) { col[off] = (int32_t)(r + 1); val[off++] = -ce + fmin(Fe, 0.0); }
				if (j + 1 < n) { col[off] = (int32_t)(r + n); val[off++] = -cn + fmin(Fn, 0.0); }
				if (k + 1 < n) { col[off] = (int32_t)(r + n2); val[off++] = -ct + fmin(Ft, 0.0); }
				rowptr[r + 1] = off;
			}
	if (!vel)
		free(u);
}
