// Staged CGS2 orthogonalisation of the new Arnoldi vector v against the basis
// V_0..V_k (kp1 = k + 1 <= kStagedMax vectors), three passes over the basis,
// one launch each:
//   pass 1: h1 = V^T v
//   pass 2: v' = v - V h1 (in registers, not stored), h2 = V^T v' and
//           ||v'||^2; the last CTA forms the Hessenberg column h1 + h2 and
//           ||v''||, v'' = v' - V h2, as sqrt(||v'||^2 - ||h2||^2) (V has
//           orthonormal columns, so V^T V h2 = h2 up to rounding), then
//           finishes the step (rotations, residual estimate, stop / restart)
//   pass 3: V_{k+1} = (v - V (h1 + h2)) * (1 / ||v''||), or unscaled when
//           ||v''|| == 0: the normalisation of gmres.hh:156-162 folded into
//           the last update; skipped once the step stopped or restarts.
//
// Delayed CGS2 (Swirydowicz, Langou, Ananthan, Yang, Thomas, "Low
// synchronization Gram-Schmidt and generalized minimal residual algorithms",
// NLAA 28, 2021; the DCGS2 Arnoldi of Bielich, Langou, Thomas, Swirydowicz,
// Yamazaki, Boman, Parallel Computing 112, 2022): the reorthogonalisation of
// a vector is deferred to the next step, where it shares the pass of that
// step's projection, so a step costs two passes over the basis, not three.
// Column k holds u_k, the once-orthogonalised, unnormalised candidate for
// q_k; the SpMV gives w = M u_k.  With Q = q_0..q_{k-1}:
//   pass 4: t = Q^T w, gamma = u_k^T w, s = Q^T u_k, alpha = u_k^T u_k; the
//           last CTA forms r = sqrt(alpha - s^T s), finishes Hessenberg
//           column k - 1 (its tentative entries + s, and r below them:
//           M q_{k-1} = Q (h_{k-1} + s) + r q_k), then tau = q_k^T w =
//           (gamma - s^T t) / r and the tentative column k,
//           h_k = Q_k^T M q_k = ([t; tau] - H s) / r, from the Arnoldi
//           relation M Q = Q_k H;
//   pass 5: q_k = (u_k - Q s) / r over column k, and the next candidate
//           u_{k+1} = (w - Q t - tau q_k) / r into column k + 1;
//   pass 6: at the end of a cycle, s = Q^T u_m and alpha finish column m - 1.
// Step 0 starts from the normalised q_0 (r = 1, no s).  The convergence test
// of column k - 1 runs in step k's pass 4, one SpMV later than in CGS2.
//
// Data movement.  Each pass streams tiles of v and of every basis vector into
// a ring of shared-memory stages, issued by one producer lane as soon as the
// consumers have released the stage on its `empty` mbarrier and completing on
// the stage's `full` mbarrier: v with a bulk copy (cp.async.bulk), the basis
// with 2-D tensor copies (cp.async.bulk.tensor) through tensor maps of the
// basis whose boxes are kOT 8-byte elements (512 FP32 or 256 FP64 rows) by 8,
// 4, 2 or 1 columns, so that a tile of kp1 vectors takes at most six copies
// and reads no column past kp1 - 1 (a copy per 1 KB vector tile left the
// producer issuing copies and the passes at a third of HBM bandwidth; boxes
// of 8 columns only would read up to 7 unused columns).  Rows past n are
// zero-filled by the tensor unit.  A stage is kp1 + 1 slots of 2 KB; the
// ring takes up to kOSmemBudget bytes, so an SM keeps up to ~200 KB of loads
// in flight whatever kp1 is.
//
// Arithmetic.  Consumer thread t owns element t of every tile: two adjacent
// FP32 rows, summed with packed two-lane FMAs (fma.rn.f32x2), or one FP64
// row.  Its dot products accumulate per row in T across the tiles of its
// CTA; the CTA and grid folds are FP64, in a fixed order.  One CTA per SM
// (the ring fills the SM's shared memory).  Every wait is bounded: past the
// limit the CTA records an error in the context's device error word and
// winds down, and the producer waits (bounded) for its copies in flight
// before the CTA exits.
#pragma once

#include <cuda.h>

namespace fsg {
namespace {

constexpr int kOT = 256;                 // 8-byte elements per tile, one per consumer thread
constexpr int kOCons = kOT / 32;         // consumer warps
constexpr int kOThreads = kOT + 32;      // plus the producer warp
constexpr int kOWarps = kOThreads / 32;
constexpr int kOMaxStages = 32;
constexpr int kStagedMax = 31;           // basis vectors the staged passes take
constexpr int kOSlot = kOT * 8;          // bytes of one vector's tile
constexpr int kOMaps = 4;                // box heights 8, 4, 2, 1
constexpr size_t kOSmemBudget = 200 * 1024;
static_assert(kStagedMax + 1 <= kPartPerBlock, "pass 2 writes kp1 + 1 partials per CTA");
static_assert(2 * kStagedMax <= 8 * kPartPerBlock, "pass 4 writes 2 kp1 partials per CTA");
static_assert(kStagedMax + 1 <= kGmDelayedCols, "delayed CGS2 Hessenberg columns");

// the tensor maps of one basis: box heights 8, 4, 2 and 1 columns
struct BasisMaps {
	CUtensorMap m[kOMaps];
};

template<class T>
struct OrthoArgs {
	const T *v;       // the new vector (A z or D^-1 A V_k); pass 6: u_m
	T *out;           // pass 3: V_{k+1}; pass 5: u_{k+1}
	T *outq;          // pass 5: q_k (column k)
	int64_t n;
	int kp1;
	int stages;
	unsigned stride;  // bytes per stage: (kp1 + 1) slots
	GmState *g;
	KState *st;
	double *part;
	unsigned *counter;
	double *hist;
	unsigned *err;
};

inline unsigned staged_stride(int kp1) { return (unsigned)((kp1 + 1) * kOSlot); }
inline int staged_stages(int kp1) {
	const size_t s = kOSmemBudget / staged_stride(kp1);
	return (int)std::max<size_t>(2, std::min<size_t>(kOMaxStages, s));
}

// The per-thread element: two FP32 rows (packed FMA) or one FP64 row
template<class T>
struct Elem;
template<>
struct Elem<float> {
	using E = float2;
	static constexpr int R = 2;
	__device__ static E zero() { return make_float2(0.f, 0.f); }
	__device__ static E splat(float a) { return make_float2(a, a); }
	__device__ static E fma(E a, E b, E c) {
		uint64_t d;
		asm("fma.rn.f32x2 %0, %1, %2, %3;"
		    : "=l"(d)
		    : "l"(*reinterpret_cast<const uint64_t *>(&a)), "l"(*reinterpret_cast<const uint64_t *>(&b)),
		      "l"(*reinterpret_cast<const uint64_t *>(&c)));
		return *reinterpret_cast<E *>(&d);
	}
	__device__ static E mul(E a, float s) { return make_float2(a.x * s, a.y * s); }
	__device__ static double sum(E a) { return (double)a.x + (double)a.y; }
	// rows e R .. e R + R - 1 of out, those below n
	__device__ static void store(float *out, int64_t e, int64_t n, E w) {
		const int64_t r = 2 * e;
		if (r + 1 < n)
			*reinterpret_cast<float2 *>(out + r) = w;
		else if (r < n)
			out[r] = w.x;
	}
};
template<>
struct Elem<double> {
	using E = double;
	static constexpr int R = 1;
	__device__ static E zero() { return 0.0; }
	__device__ static E splat(double a) { return a; }
	__device__ static E fma(E a, E b, E c) { return ::fma(a, b, c); }
	__device__ static E mul(E a, double s) { return a * s; }
	__device__ static double sum(E a) { return a; }
	__device__ static void store(double *out, int64_t e, int64_t n, E w) {
		if (e < n)
			out[e] = w;
	}
};

// per-CTA sums of the first nv of NV per-thread values -> part[b * nv + j]
template<int NV>
__device__ __forceinline__ void staged_block_sum(const double (&vals)[NV], int nv, double *part,
                                                 double *sh) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for (int j = 0; j < NV; ++j) {
		if (j < nv) {
			double v = vals[j];
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
				v += __shfl_down_sync(0xffffffffu, v, o);
			if (lane == 0)
				sh[j * kOWarps + wid] = v;
		}
	}
	__syncthreads();
	if ((int)threadIdx.x < nv) {
		double t = 0.0;
#pragma unroll
		for (int w = 0; w < kOWarps; ++w)
			t += sh[threadIdx.x * kOWarps + w];
		part[(size_t)blockIdx.x * nv + threadIdx.x] = t;
	}
}

// last CTA: out[j] = sum over CTAs of part[b * nv + j], j < nv <= 32.  Warp
// c sums the CTAs c, c + kOWarps, ... in order (lane j: value j, so a warp
// reads contiguous partials), then the kOWarps sums are added in order.
__device__ __forceinline__ void staged_fold(const double *part, int nv, double *out, double *sh) {
	const int j = threadIdx.x & 31, c = threadIdx.x >> 5;
	double t = 0.0;
	if (j < nv)
		for (unsigned b = c; b < gridDim.x; b += kOWarps)
			t += __ldcg(part + (size_t)b * nv + j);
	__syncthreads();  // sh was used by the CTA's own sum
	sh[c * 32 + j] = t;
	__syncthreads();
	if ((int)threadIdx.x < nv) {
		double s = 0.0;
#pragma unroll
		for (int w = 0; w < kOWarps; ++w)
			s += sh[w * 32 + threadIdx.x];
		out[threadIdx.x] = s;
	}
	__syncthreads();
}

// 2-D tensor copy of the box at (element c0, column c1) into shared memory,
// completing on `bar` (the full box's bytes, zero-filled past the tensor)
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            unsigned long long *bar) {
	asm volatile(
		"cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
		" [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_addr(dst)),
		"l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
		: "memory");
}

template<class T, int NA, int PASS>
__global__ void __launch_bounds__(kOThreads, 1)
k_gm_staged(OrthoArgs<T> a, const __grid_constant__ BasisMaps maps) {
	static_assert(NA % 8 == 0 && NA <= 32, "accumulator slots");
	using EL = Elem<T>;
	using E = typename EL::E;
	constexpr int R = EL::R;  // rows per element
	extern __shared__ __align__(128) unsigned char smem_dyn[];
	// tensor copies land on 128-byte boundaries
	unsigned char *smem_raw = reinterpret_cast<unsigned char *>(
		(reinterpret_cast<uintptr_t>(smem_dyn) + 127) & ~(uintptr_t)127);
	__shared__ unsigned long long full[kOMaxStages], empty[kOMaxStages];
	__shared__ T hs[kStagedMax + 1], ht[kStagedMax + 1];
	__shared__ double sh[32 * kOWarps];
	__shared__ double folded[64];
	__shared__ int abort_flag;
	if (stopped(a.st))
		return;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int kp1 = a.kp1, S = a.stages;
	const int64_t nelem = (a.n + R - 1) / R;
	const int64_t ntile = (nelem + kOT - 1) / kOT;
	const int nt = ntile > (int64_t)blockIdx.x ? (int)((ntile - 1 - blockIdx.x) / gridDim.x + 1) : 0;
	if (tid == 0) {
		abort_flag = 0;
		for (int s = 0; s < S; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], kOCons);
		}
		mbar_init_fence();
	}
	double vn = 0.0;
	if constexpr (PASS == 2) {
		for (int j = tid; j < kp1; j += blockDim.x)
			hs[j] = (T)a.g->h1[j];
	}
	if constexpr (PASS == 3) {
		for (int j = tid; j < kp1; j += blockDim.x)
			hs[j] = (T)(a.g->h1[j] + a.g->h2[j]);
		vn = a.g->vnorm;
	}
	double tau = 0.0;
	if constexpr (PASS == 5) {
		for (int j = tid; j < kp1 - 1; j += blockDim.x) {
			hs[j] = (T)a.g->h1[j];
			ht[j] = (T)a.g->h2[j];
		}
		vn = a.g->dg_r;
		tau = a.g->dg_tau;
	}
	__syncthreads();
	volatile int *abort_v = &abort_flag;
	E acc[NA];
#pragma unroll
	for (int j = 0; j < NA; ++j)
		acc[j] = EL::zero();
	E accn = EL::zero();
	if (warp == kOCons) {
		// producer: one lane issues every copy of a tile
		if (lane == 0) {
			int issued = 0;
			for (int i = 0; i < nt; ++i) {
				const int s = i % S;
				if (i >= S && !mbar_wait(&empty[s], (unsigned)(((i / S) - 1) & 1))) {
					atomicOr(a.err, 1u);
					*abort_v = 1;
					break;
				}
				if (*abort_v)
					break;
				const int64_t e0 = ((int64_t)blockIdx.x + (int64_t)i * gridDim.x) * kOT;
				const int64_t r0 = e0 * R;
				const int64_t rows = a.n - r0 < (int64_t)kOT * R ? a.n - r0 : (int64_t)kOT * R;
				// 16-byte multiple; the tail reads into v's padding
				const unsigned bytes = (unsigned)((rows * (int64_t)sizeof(T) + 15) & ~(int64_t)15);
				unsigned char *dst = smem_raw + (size_t)s * a.stride;
				mbar_arrive_expect_tx(&full[s], bytes + (unsigned)kp1 * kOSlot);
				bulk_g2s(dst, a.v + r0, bytes, &full[s]);
				// columns 0 .. kp1 - 1: boxes of 8 while 8 remain, then at
				// most one box each of 4, 2 and 1
				int c = 0;
				while (kp1 - c >= 8) {
					tma_load_2d(dst + (size_t)(1 + c) * kOSlot, &maps.m[0], (int)e0, c, &full[s]);
					c += 8;
				}
#pragma unroll
				for (int m = 1; m < kOMaps; ++m) {
					const int h = 8 >> m;
					if (kp1 - c >= h) {
						tma_load_2d(dst + (size_t)(1 + c) * kOSlot, &maps.m[m], (int)e0, c, &full[s]);
						c += h;
					}
				}
				issued = i + 1;
			}
			// every copy lands before the CTA exits
			for (int j = issued > S ? issued - S : 0; j < issued; ++j)
				mbar_wait(&full[j % S], (unsigned)((j / S) & 1));
		}
	}
	else {
		const T inv = (T)(vn != 0.0 ? 1.0 / vn : 1.0);
		for (int i = 0; i < nt; ++i) {
			const int s = i % S;
			if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (unsigned)((i / S) & 1)))) {
				if (lane == 0) {
					atomicOr(a.err, 1u);
					*abort_v = 1;
				}
				break;
			}
			const E *sv = reinterpret_cast<const E *>(smem_raw + (size_t)s * a.stride);
			const int64_t tile0 = ((int64_t)blockIdx.x + (int64_t)i * gridDim.x) * kOT;
			const int64_t e = tile0 + tid;
			if constexpr (PASS == 4) {
				// the consumers in two halves: warps 0-3 sum w . V_j, warps
				// 4-7 u_k . V_j (u_k is column k = kp1 - 1), each thread over
				// elements lt and lt + kOT / 2 of the tile -- one set of
				// accumulators a thread, as in pass 1
				const int lt = tid & (kOT / 2 - 1), grp = tid / (kOT / 2);
				const int xslot = grp == 0 ? 0 : kp1;
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					const int el = lt + h * (kOT / 2);
					if (tile0 + el < nelem) {
						const E xv = sv[xslot * kOT + el];
#pragma unroll
						for (int j = 0; j < NA; ++j)
							if (j < kp1)
								acc[j] = EL::fma(xv, sv[(j + 1) * kOT + el], acc[j]);
					}
				}
			}
			else if (e < nelem) {
				const E vi = sv[tid];
				if constexpr (PASS == 1 || PASS == 6) {
#pragma unroll
					for (int j = 0; j < NA; ++j)
						if (j < kp1)
							acc[j] = EL::fma(vi, sv[(j + 1) * kOT + tid], acc[j]);
				}
				else if constexpr (PASS == 5) {
					const int k = kp1 - 1;
					const E ui = sv[kp1 * kOT + tid];
					E q = ui, u1 = vi;
#pragma unroll
					for (int j = 0; j < NA; ++j)
						if (j < k) {
							const E vj = sv[(j + 1) * kOT + tid];
							q = EL::fma(EL::splat(-hs[j]), vj, q);
							u1 = EL::fma(EL::splat(-ht[j]), vj, u1);
						}
					if (k > 0) {
						q = EL::mul(q, inv);
						EL::store(a.outq, e, a.n, q);
					}
					u1 = EL::fma(EL::splat((T)-tau), q, u1);
					EL::store(a.out, e, a.n, EL::mul(u1, inv));
				}
				else {
					E w = vi;
#pragma unroll
					for (int j = 0; j < NA; ++j)
						if (j < kp1)
							w = EL::fma(EL::splat(-hs[j]), sv[(j + 1) * kOT + tid], w);
					if constexpr (PASS == 2) {
#pragma unroll
						for (int j = 0; j < NA; ++j)
							if (j < kp1)
								acc[j] = EL::fma(w, sv[(j + 1) * kOT + tid], acc[j]);
						accn = EL::fma(w, w, accn);
					}
					else {
						EL::store(a.out, e, a.n, vn != 0.0 ? EL::mul(w, inv) : w);
					}
				}
			}
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&empty[s]);
			if (__any_sync(0xffffffffu, *abort_v != 0))
				break;
		}
	}
	if constexpr (PASS == 4 || PASS == 6) {
		// pass 4: t and gamma (kp1 values, the first half of the consumers),
		// then s and alpha (kp1 values, the second half) in a second block of
		// partials; pass 6: s and alpha
		const int grp = tid / (kOT / 2);
		double vals[NA];
#pragma unroll
		for (int j = 0; j < NA; ++j)
			vals[j] = j < kp1 && (PASS == 6 || grp == 0) ? EL::sum(acc[j]) : 0.0;
		staged_block_sum<NA>(vals, kp1, a.part, sh);
		double *part2 = a.part + (size_t)gridDim.x * kp1;
		if constexpr (PASS == 4) {
#pragma unroll
			for (int j = 0; j < NA; ++j)
				vals[j] = j < kp1 && grp == 1 ? EL::sum(acc[j]) : 0.0;
			__syncthreads();  // sh of the first sum is read
			staged_block_sum<NA>(vals, kp1, part2, sh);
		}
		if (last_block(a.counter)) {
			staged_fold(a.part, kp1, folded, sh);
			if constexpr (PASS == 4)
				staged_fold(part2, kp1, folded + 32, sh);
			// the scalar work, spread over the CTA where it is independent:
			// every thread forms r and tau from shared memory; thread j
			// finishes H(j, k - 1), thread i forms the tentative H(i, k)
			GmState *g = a.g;
			const int k = kp1 - 1, ldh = g->ld;
			const double *s = PASS == 4 ? folded + 32 : folded;
			const double *t = folded;
			double ss = 0.0, st_ = 0.0;
			for (int j = 0; j < k; ++j) {
				ss += s[j] * s[j];
				if constexpr (PASS == 4)
					st_ += s[j] * t[j];
			}
			const double r = k > 0 ? sqrt(fmax(s[k] - ss, 0.0)) : 1.0;
			const double rinv = r != 0.0 ? 1.0 / r : 1.0;
			if (k > 0) {
				// column k - 1 is final: its tentative entries + s, r below
				const int c = k - 1;
				if (tid < k) {
					const double hv = g->Hr[tid + kGmDelayedCols * c] + s[tid];
					g->Hr[tid + kGmDelayedCols * c] = hv;
					g->H[tid + ldh * c] = hv;
				}
				if (tid == 0) {
					g->Hr[k + kGmDelayedCols * c] = r;
					g->H[k + ldh * c] = r;
					g->vnorm = r;
				}
				__syncthreads();
				finish_step_cta(g, a.st, a.hist, sh);
			}
			if constexpr (PASS == 4) {
				const double tau_k = (t[k] - st_) * rinv;
				// tentative column k: ([t; tau] - H s) / r over rows 0..k
				if (tid <= k) {
					const int i = tid;
					double hs_i = 0.0;
#pragma unroll 8
					for (int j = i > 0 ? i - 1 : 0; j < k; ++j)
						hs_i += g->Hr[i + kGmDelayedCols * j] * s[j];
					g->Hr[i + kGmDelayedCols * k] = ((i < k ? t[i] : tau_k) - hs_i) * rinv;
				}
				if (tid < k) {
					g->h1[tid] = s[tid];
					g->h2[tid] = t[tid];
				}
				if (tid == 0) {
					g->dg_tau = tau_k;
					g->dg_r = r;
				}
			}
			if (tid == 0)
				*a.counter = 0;
		}
	}
	if constexpr (PASS == 1 || PASS == 2) {
		// pass 2 puts ||v'||^2 right after the kp1 dots
		constexpr int NS = PASS == 2 ? NA + 1 : NA;
		double vals[NS];
#pragma unroll
		for (int j = 0; j < NS; ++j) {
			const double aj = j < NA ? EL::sum(acc[j < NA ? j : 0]) : 0.0;
			vals[j] = j < kp1 ? aj : (PASS == 2 && j == kp1 ? EL::sum(accn) : 0.0);
		}
		const int nv = PASS == 2 ? kp1 + 1 : kp1;
		staged_block_sum<NS>(vals, nv, a.part, sh);
		if (last_block(a.counter)) {
			staged_fold(a.part, nv, folded, sh);
			GmState *g = a.g;
			if constexpr (PASS == 1) {
				if (tid < kp1)
					g->h1[tid] = folded[tid];
			}
			else {
				const int k = g->k, ldh = g->ld;
				if (tid < kp1) {
					g->h2[tid] = folded[tid];
					g->H[tid + ldh * k] = g->h1[tid] + folded[tid];
				}
				if (tid == 0) {
					double s2 = 0.0;
					for (int j = 0; j < kp1; ++j)
						s2 += folded[j] * folded[j];
					const double vn2 = sqrt(fmax(folded[kp1] - s2, 0.0));
					g->H[kp1 + ldh * k] = vn2;
					g->vnorm = vn2;
				}
				__syncthreads();
				finish_step_cta(g, a.st, a.hist, sh);
			}
			if (tid == 0)
				*a.counter = 0;
		}
	}
}

template<class T, int NA, int PASS>
int launch_staged(Ctx *ctx, const OrthoArgs<T> &a, const BasisMaps &maps) {
	static bool ready = false;
	auto kern = k_gm_staged<T, NA, PASS>;
	const size_t smem = (size_t)a.stages * a.stride + 128;
	if (!ready) {
		if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)(kOSmemBudget + 128)) != cudaSuccess)
			return set_err(ctx, FS_ERR_CUDA, "gmres: cannot reserve %zu bytes of shared memory",
			               kOSmemBudget + 128);
		ready = true;
	}
	kern<<<ctx->sms, kOThreads, smem, ctx->stream>>>(a, maps);
	return check_launch(ctx, "gmres staged orthogonalisation");
}

template<class T, int PASS>
int staged_pass(Ctx *ctx, const OrthoArgs<T> &a, const BasisMaps &maps) {
	switch ((a.kp1 + 7) / 8) {
	case 1: return launch_staged<T, 8, PASS>(ctx, a, maps);
	case 2: return launch_staged<T, 16, PASS>(ctx, a, maps);
	case 3: return launch_staged<T, 24, PASS>(ctx, a, maps);
	default: return launch_staged<T, 32, PASS>(ctx, a, maps);
	}
}

// The tensor maps of an ld x cols basis of T, as 8-byte elements (a pair of
// FP32 rows or one FP64 row; the copies move raw bits): elements innermost
// (ceil(n / pairs) of them; an odd FP32 n ends in the column's padding),
// columns ld * sizeof(T) bytes apart, boxes of kOT elements by 8, 4, 2 and 1
// columns, zero fill outside.  false when the driver's encoder is unavailable
// or refuses.
template<class T>
bool encode_basis_maps(BasisMaps *maps, const T *V, int64_t n, int64_t ld, int cols) {
	using encode_fn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
	                               const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
	                               const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
	                               CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
	static encode_fn fn = [] {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
		                                     &q) != cudaSuccess ||
		    q != cudaDriverEntryPointSuccess) {
			cudaGetLastError();
			p = nullptr;
		}
		return reinterpret_cast<encode_fn>(p);
	}();
	constexpr int R = 8 / (int)sizeof(T);
	if (!fn || n <= 0 || n >= ((int64_t)1 << 31) || ((uintptr_t)V & 15) || (ld * sizeof(T)) % 16 ||
	    ld < (n + R - 1) / R * R)
		return false;
	const cuuint64_t dims[2] = {(cuuint64_t)((n + R - 1) / R), (cuuint64_t)cols};
	const cuuint64_t strides[1] = {(cuuint64_t)(ld * sizeof(T))};
	const cuuint32_t estr[2] = {1, 1};
	for (int m = 0; m < kOMaps; ++m) {
		const cuuint32_t box[2] = {(cuuint32_t)kOT, (cuuint32_t)(8 >> m)};
		if (fn(&maps->m[m], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<T *>(V), dims, strides, box,
		       estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
		       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return false;
	}
	return true;
}

}  // namespace
}  // namespace fsg
