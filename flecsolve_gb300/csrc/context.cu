// Context, vector lifecycle and the vector Operations policy of the C ABI.
//
// Replaces the FleCSI-task vector backend of flecsolve
// (flecsolve/vectors/operations/topo_view.hh:26-291 dispatching the tasks of
// vectors/operations/topo_tasks.hh:35-324): each elementwise op is one
// grid-stride kernel on the context stream, each reduction is one kernel
// whose last block folds the per-block partials in a fixed order, so results
// are reproducible run to run.
#include <cmath>
#include <cstring>

#include "fsgpu_internal.cuh"

namespace fsg {

int set_err(Ctx *ctx, int status, const char *fmt, ...) {
	if (ctx && ctx->magic == kMagicCtx) {
		char buf[1024];
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(buf, sizeof buf, fmt, ap);
		va_end(ap);
		ctx->err = buf;
	}
	return status;
}

int check_device_error(Ctx *ctx) {
	unsigned *h = reinterpret_cast<unsigned *>(ctx->host_out + 15);
	FS_CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->dev_err, sizeof(unsigned), cudaMemcpyDeviceToHost,
	                                 ctx->stream));
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	if (*h) {
		const unsigned e = *h;
		*h = 0;
		FS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->dev_err, 0, sizeof(unsigned), ctx->stream));
		return set_err(ctx, FS_ERR_CUDA, "a device-side wait ran out of its iteration limit (code %u)", e);
	}
	return FS_OK;
}

int check_launch(Ctx *ctx, const char *what) {
	ctx->launches++;
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess)
		return set_err(ctx, FS_ERR_CUDA, "launch of %s failed: %s", what,
		               cudaGetErrorString(e));
	return FS_OK;
}

// every elementwise / reduction grid is at most 8 CTAs per SM; the solver
// partials buffers are sized on that bound
int grid_for(Ctx *ctx, int64_t n, int threads, int per_thread) {
	int64_t want = (n + (int64_t)threads * per_thread - 1) / ((int64_t)threads * per_thread);
	int64_t cap = (int64_t)ctx->sms * 8;
	if (want < 1)
		want = 1;
	return (int)(want < cap ? want : cap);
}

// ------------------------------------------------ elementwise kernels --

enum EwOp {
	EW_COPY, EW_SET, EW_SCALE, EW_ADD, EW_SUB, EW_MUL, EW_DIV, EW_RECIP,
	EW_LINSUM, EW_AXPY, EW_AXPBY, EW_ABS, EW_ADDS
};

template<class T, int OP>
__global__ void ew_kernel(int64_t n, T a, T b, const T *x, const T *y, T *z) {
	// no __restrict__: the output may alias an input (in-place variants of
	// operations/topo_view.hh:78-210); each index is read before it is written
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x) {
		T r;
		if constexpr (OP == EW_COPY) r = x[i];
		else if constexpr (OP == EW_SET) r = a;
		else if constexpr (OP == EW_SCALE) r = a * x[i];
		else if constexpr (OP == EW_ADD) r = x[i] + y[i];
		else if constexpr (OP == EW_SUB) r = x[i] - y[i];
		else if constexpr (OP == EW_MUL) r = x[i] * y[i];
		else if constexpr (OP == EW_DIV) r = x[i] / y[i];
		else if constexpr (OP == EW_RECIP) r = T(1) / x[i];
		else if constexpr (OP == EW_LINSUM) r = a * x[i] + b * y[i];
		else if constexpr (OP == EW_AXPY) r = a * x[i] + y[i];
		else if constexpr (OP == EW_AXPBY) r = a * x[i] + b * y[i];
		else if constexpr (OP == EW_ABS) r = x[i] < T(0) ? -x[i] : x[i];
		else r = x[i] + a;
		z[i] = r;
	}
}

__device__ __forceinline__ double u01_at(uint64_t seed, uint64_t i) {
	// splitmix64 of (seed, index): counter-based so the kernel is order free
	uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	z ^= z >> 31;
	return (double)(z >> 11) * 0x1.0p-53;
}

template<class T>
__global__ void rand_kernel(int64_t n, uint64_t seed, T *z) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x)
		z[i] = (T)u01_at(seed, (uint64_t)i);
}

template<class T, int OP>
static int ew_launch(Ctx *ctx, int64_t n, double a, double b, const void *x,
                     const void *y, void *z) {
	if (n == 0)
		return FS_OK;
	int g = grid_for(ctx, n, 256, 4);
	ew_kernel<T, OP><<<g, 256, 0, ctx->stream>>>(n, (T)a, (T)b, (const T *)x,
	                                            (const T *)y, (T *)z);
	return check_launch(ctx, "vector op");
}

template<int OP>
static int ew(Vec *z, double a, double b, Vec *x, Vec *y) {
	if (!ok_vec(z) || (x && !ok_vec(x)) || (y && !ok_vec(y)))
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = z->ctx;
	if ((x && (x->n != z->n || x->dtype != z->dtype)) ||
	    (y && (y->n != z->n || y->dtype != z->dtype)))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH,
		               "vector op: sizes or dtypes differ");
	if (z->dtype == FS_F64)
		return ew_launch<double, OP>(ctx, z->n, a, b, x ? x->d : nullptr,
		                             y ? y->d : nullptr, z->d);
	return ew_launch<float, OP>(ctx, z->n, a, b, x ? x->d : nullptr,
	                            y ? y->d : nullptr, z->d);
}

// -------------------------------------------------------- reductions --

enum RedOp { RD_DOT, RD_L1, RD_INF, RD_MIN, RD_MAX };

// One kernel per reduction: per-thread fixed strided partials, block tree,
// per-block partial to `part`, last block folds the partials in block order.
template<int OP>
__global__ void __launch_bounds__(kRedThreads)
red_f64(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
        double *part, double *out, unsigned *counter) {
	__shared__ double sh[32];
	double acc[1];
	if constexpr (OP == RD_MIN) acc[0] = INFINITY;
	else if constexpr (OP == RD_MAX) acc[0] = -INFINITY;
	else acc[0] = 0.0;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x) {
		double v = x[i];
		if constexpr (OP == RD_DOT) acc[0] = fma(v, y[i], acc[0]);
		else if constexpr (OP == RD_L1) acc[0] += fabs(v);
		else if constexpr (OP == RD_INF) acc[0] = fmax(acc[0], fabs(v));
		else if constexpr (OP == RD_MIN) acc[0] = fmin(acc[0], v);
		else acc[0] = fmax(acc[0], v);
	}
	if constexpr (OP == RD_DOT || OP == RD_L1) {
		block_sum<1>(acc, sh);
	}
	else {
		for (int o = 16; o > 0; o >>= 1) {
			double t = __shfl_down_sync(0xffffffffu, acc[0], o);
			acc[0] = (OP == RD_MIN) ? fmin(acc[0], t) : fmax(acc[0], t);
		}
		__syncthreads();
		if ((threadIdx.x & 31) == 0)
			sh[threadIdx.x >> 5] = acc[0];
		__syncthreads();
		if (threadIdx.x == 0)
			for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
				acc[0] = (OP == RD_MIN) ? fmin(acc[0], sh[w]) : fmax(acc[0], sh[w]);
	}
	if (threadIdx.x == 0)
		part[blockIdx.x] = acc[0];
	if (last_block(counter)) {
		double r[1];
		if constexpr (OP == RD_DOT || OP == RD_L1) {
			sum_partials<1>(part, gridDim.x, r, sh);
		}
		else {
			r[0] = __ldcg(part);
			if (threadIdx.x == 0)
				for (unsigned b = 1; b < gridDim.x; ++b) {
					double t = __ldcg(part + b);
					r[0] = (OP == RD_MIN) ? fmin(r[0], t) : fmax(r[0], t);
				}
		}
		if (threadIdx.x == 0) {
			*out = r[0];
			*counter = 0;
		}
	}
}

template<int OP>
__global__ void __launch_bounds__(kRedThreads)
red_f32(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
        double *part, double *out, unsigned *counter) {
	__shared__ float shf[64];
	__shared__ double sh[32];
	if constexpr (OP == RD_DOT || OP == RD_L1) {
		cf32 acc[1] = {{0.f, 0.f}};
		for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
		     i += (int64_t)gridDim.x * blockDim.x) {
			if constexpr (OP == RD_DOT) acc[0].add_prod(x[i], y[i]);
			else acc[0].add(fabsf(x[i]));
		}
		block_sum_cf<1>(acc, shf);
		if (threadIdx.x == 0)
			part[blockIdx.x] = (double)acc[0].hi + (double)acc[0].lo;
	}
	else {
		float a = (OP == RD_MIN) ? INFINITY : (OP == RD_MAX ? -INFINITY : 0.f);
		for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
		     i += (int64_t)gridDim.x * blockDim.x) {
			float v = x[i];
			if constexpr (OP == RD_INF) a = fmaxf(a, fabsf(v));
			else if constexpr (OP == RD_MIN) a = fminf(a, v);
			else a = fmaxf(a, v);
		}
		for (int o = 16; o > 0; o >>= 1) {
			float t = __shfl_down_sync(0xffffffffu, a, o);
			a = (OP == RD_MIN) ? fminf(a, t) : fmaxf(a, t);
		}
		__syncthreads();
		if ((threadIdx.x & 31) == 0)
			shf[threadIdx.x >> 5] = a;
		__syncthreads();
		if (threadIdx.x == 0) {
			for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
				a = (OP == RD_MIN) ? fminf(a, shf[w]) : fmaxf(a, shf[w]);
			part[blockIdx.x] = a;
		}
	}
	if (last_block(counter)) {
		double r[1];
		if constexpr (OP == RD_DOT || OP == RD_L1) {
			sum_partials<1>(part, gridDim.x, r, sh);
		}
		else {
			r[0] = __ldcg(part);
			if (threadIdx.x == 0)
				for (unsigned b = 1; b < gridDim.x; ++b) {
					double t = __ldcg(part + b);
					r[0] = (OP == RD_MIN) ? fmin(r[0], t) : fmax(r[0], t);
				}
		}
		if (threadIdx.x == 0) {
			*out = r[0];
			*counter = 0;
		}
	}
}

template<int OP>
static int reduce(Vec *x, Vec *y, double *out) {
	if (!ok_vec(x) || (y && !ok_vec(y)))
		return FS_ERR_BAD_HANDLE;
	if (!out)
		return FS_ERR_INVALID_ARG;
	Ctx *ctx = x->ctx;
	if (y && (y->n != x->n || y->dtype != x->dtype))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "reduction: sizes or dtypes differ");
	int g = grid_for(ctx, x->n, kRedThreads, 8);
	if (x->dtype == FS_F64)
		red_f64<OP><<<g, kRedThreads, 0, ctx->stream>>>(
			x->n, (const double *)x->d, y ? (const double *)y->d : nullptr,
			ctx->red_part, ctx->red_out, ctx->red_count);
	else
		red_f32<OP><<<g, kRedThreads, 0, ctx->stream>>>(
			x->n, (const float *)x->d, y ? (const float *)y->d : nullptr,
			ctx->red_part, ctx->red_out, ctx->red_count);
	FS_TRY(check_launch(ctx, "reduction"));
	FS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->host_out, ctx->red_out, sizeof(double),
	                                 cudaMemcpyDeviceToHost, ctx->stream));
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	*out = *ctx->host_out;
	return FS_OK;
}

}  // namespace fsg

using namespace fsg;

// ================================================================ C ABI ==

extern "C" {

FS_API const char *fs_status_string(int s) {
	switch (s) {
	case FS_OK: return "ok";
	case FS_ERR_BAD_HANDLE: return "bad handle";
	case FS_ERR_SIZE_MISMATCH: return "size mismatch";
	case FS_ERR_OUT_OF_MEMORY: return "out of device memory";
	case FS_ERR_CUDA: return "CUDA error";
	case FS_ERR_NON_FINITE: return "non-finite value";
	case FS_ERR_BREAKDOWN: return "solver breakdown";
	case FS_ERR_INVALID_ARG: return "invalid argument";
	case FS_ERR_NO_DEVICE: return "no CUDA device";
	case FS_ERR_UNSUPPORTED: return "unsupported";
	case FS_ERR_IO: return "file missing, unreadable or malformed";
	default: return "unknown status";
	}
}

FS_API int fs_ctx_create(int device, fs_ctx *out) {
	if (!out)
		return FS_ERR_INVALID_ARG;
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
		cudaGetLastError();
		return FS_ERR_NO_DEVICE;
	}
	if (device < 0 || device >= ndev)
		return FS_ERR_INVALID_ARG;
	if (cudaSetDevice(device) != cudaSuccess)
		return FS_ERR_CUDA;
	Ctx *c = new Ctx();
	c->device = device;
	cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
	auto fail = [&](int st) {
		if (c->stream) cudaStreamDestroy(c->stream);
		if (c->red_part) cudaFree(c->red_part);
		if (c->red_out) cudaFree(c->red_out);
		if (c->red_count) cudaFree(c->red_count);
		if (c->host_out) cudaFreeHost(c->host_out);
		delete c;
		return st;
	};
	if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
		return fail(FS_ERR_CUDA);
	if (cudaMalloc(&c->red_part, sizeof(double) * kMaxRedBlocks * 4) != cudaSuccess ||
	    cudaMalloc(&c->red_out, sizeof(double) * 8) != cudaSuccess ||
	    cudaMalloc(&c->red_count, sizeof(unsigned) * 16) != cudaSuccess ||
	    cudaMallocHost(&c->host_out, sizeof(double) * 16) != cudaSuccess)
		return fail(FS_ERR_OUT_OF_MEMORY);
	c->dev_err = c->red_count + 15;
	if (cudaMemset(c->red_count, 0, sizeof(unsigned) * 16) != cudaSuccess ||
	    fence_setup_copies() != cudaSuccess)
		return fail(FS_ERR_CUDA);
	*out = reinterpret_cast<fs_ctx>(c);
	return FS_OK;
}

FS_API int fs_ctx_destroy(fs_ctx h) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c))
		return FS_ERR_BAD_HANDLE;
	cudaSetDevice(c->device);
	cudaStreamSynchronize(c->stream);
	for (auto &e : c->ev)
		if (e)
			cudaEventDestroy(e);
	cudaFree(c->red_part);
	cudaFree(c->red_out);
	cudaFree(c->red_count);
	cudaFreeHost(c->host_out);
	cudaStreamDestroy(c->stream);
	c->magic = 0;
	delete c;
	return FS_OK;
}

FS_API int fs_ctx_sync(fs_ctx h) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c))
		return FS_ERR_BAD_HANDLE;
	FS_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
	return check_device_error(c);
}

FS_API int fs_ctx_stream(fs_ctx h, void **stream) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !stream)
		return FS_ERR_BAD_HANDLE;
	*stream = (void *)c->stream;
	return FS_OK;
}

FS_API int fs_ctx_sm_count(fs_ctx h, int *sms) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !sms)
		return FS_ERR_BAD_HANDLE;
	*sms = c->sms;
	return FS_OK;
}

FS_API const char *fs_last_error(fs_ctx h) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c))
		return "bad context handle";
	return c->err.c_str();
}

FS_API int fs_ctx_launch_count(fs_ctx h, int64_t *count) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !count)
		return FS_ERR_BAD_HANDLE;
	*count = c->launches;
	return FS_OK;
}

FS_API int fs_ctx_event_record(fs_ctx h, int slot) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c))
		return FS_ERR_BAD_HANDLE;
	if (slot < 0 || slot >= 16)
		return set_err(c, FS_ERR_INVALID_ARG, "event slot %d out of range", slot);
	if (!c->ev[slot])
		FS_CUDA_TRY(c, cudaEventCreate(&c->ev[slot]));
	FS_CUDA_TRY(c, cudaEventRecord(c->ev[slot], c->stream));
	return FS_OK;
}

FS_API int fs_ctx_event_elapsed(fs_ctx h, int a, int b, float *ms) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !ms)
		return FS_ERR_BAD_HANDLE;
	if (a < 0 || a >= 16 || b < 0 || b >= 16 || !c->ev[a] || !c->ev[b])
		return set_err(c, FS_ERR_INVALID_ARG, "event slots not recorded");
	FS_CUDA_TRY(c, cudaEventSynchronize(c->ev[b]));
	FS_CUDA_TRY(c, cudaEventElapsedTime(ms, c->ev[a], c->ev[b]));
	return FS_OK;
}

// ------------------------------------------------------------ vectors --

FS_API int fs_vec_create(fs_ctx h, int64_t n, int dtype, fs_vec *out) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !out)
		return FS_ERR_BAD_HANDLE;
	if (n < 0 || (dtype != FS_F64 && dtype != FS_F32))
		return set_err(c, FS_ERR_INVALID_ARG, "fs_vec_create: bad size or dtype");
	Vec *v = new Vec();
	v->ctx = c;
	v->n = n;
	v->dtype = dtype;
	// pad to 32 elements so vectorised accesses never leave the allocation
	size_t bytes = (size_t)((n + 31) / 32 * 32) * (dtype == FS_F64 ? 8 : 4);
	if (bytes == 0)
		bytes = 256;
	cudaError_t e = cudaMalloc(&v->d, bytes);
	if (e != cudaSuccess) {
		delete v;
		cudaGetLastError();
		return set_err(c, FS_ERR_OUT_OF_MEMORY, "fs_vec_create: %s", cudaGetErrorString(e));
	}
	cudaMemsetAsync(v->d, 0, bytes, c->stream);
	*out = reinterpret_cast<fs_vec>(v);
	return FS_OK;
}

FS_API int fs_vec_wrap(fs_ctx h, int64_t n, int dtype, void *dptr, fs_vec *out) {
	Ctx *c = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(c) || !out)
		return FS_ERR_BAD_HANDLE;
	if (n < 0 || (dtype != FS_F64 && dtype != FS_F32) || (!dptr && n > 0))
		return set_err(c, FS_ERR_INVALID_ARG, "fs_vec_wrap: bad arguments");
	Vec *v = new Vec();
	v->ctx = c;
	v->n = n;
	v->dtype = dtype;
	v->d = dptr;
	v->owns = false;
	*out = reinterpret_cast<fs_vec>(v);
	return FS_OK;
}

FS_API int fs_vec_destroy(fs_vec h) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v))
		return FS_ERR_BAD_HANDLE;
	if (v->owns && v->d) {
		cudaStreamSynchronize(v->ctx->stream);
		cudaFree(v->d);
	}
	v->magic = 0;
	delete v;
	return FS_OK;
}

FS_API int fs_vec_size(fs_vec h, int64_t *n) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v) || !n)
		return FS_ERR_BAD_HANDLE;
	*n = v->n;
	return FS_OK;
}

FS_API int fs_vec_dtype(fs_vec h, int *dt) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v) || !dt)
		return FS_ERR_BAD_HANDLE;
	*dt = v->dtype;
	return FS_OK;
}

FS_API int fs_vec_device_ptr(fs_vec h, void **p) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v) || !p)
		return FS_ERR_BAD_HANDLE;
	*p = v->d;
	return FS_OK;
}

FS_API int fs_vec_upload(fs_vec h, const void *host, int64_t n) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v))
		return FS_ERR_BAD_HANDLE;
	if (n != v->n || (!host && n > 0))
		return set_err(v->ctx, FS_ERR_SIZE_MISMATCH, "fs_vec_upload: %lld != %lld",
		               (long long)n, (long long)v->n);
	if (n == 0)
		return FS_OK;
	FS_CUDA_TRY(v->ctx, cudaMemcpyAsync(v->d, host, v->bytes(), cudaMemcpyHostToDevice,
	                                    v->ctx->stream));
	FS_CUDA_TRY(v->ctx, cudaStreamSynchronize(v->ctx->stream));
	return FS_OK;
}

FS_API int fs_vec_download(fs_vec h, void *host, int64_t n) {
	Vec *v = reinterpret_cast<Vec *>(h);
	if (!ok_vec(v))
		return FS_ERR_BAD_HANDLE;
	if (n != v->n || (!host && n > 0))
		return set_err(v->ctx, FS_ERR_SIZE_MISMATCH, "fs_vec_download: %lld != %lld",
		               (long long)n, (long long)v->n);
	if (n == 0)
		return FS_OK;
	FS_CUDA_TRY(v->ctx, cudaMemcpyAsync(host, v->d, v->bytes(), cudaMemcpyDeviceToHost,
	                                    v->ctx->stream));
	FS_CUDA_TRY(v->ctx, cudaStreamSynchronize(v->ctx->stream));
	return FS_OK;
}

#define V(h) reinterpret_cast<Vec *>(h)

FS_API int fs_vec_copy(fs_vec src, fs_vec dst) {
	if (!ok_vec(V(src)) || !ok_vec(V(dst)))
		return FS_ERR_BAD_HANDLE;
	if (src == dst)
		return FS_OK;
	return ew<EW_COPY>(V(dst), 0, 0, V(src), nullptr);
}
FS_API int fs_vec_zero(fs_vec x) { return ew<EW_SET>(V(x), 0.0, 0, nullptr, nullptr); }
FS_API int fs_vec_set_scalar(fs_vec x, double a) { return ew<EW_SET>(V(x), a, 0, nullptr, nullptr); }
FS_API int fs_vec_scale(double a, fs_vec x, fs_vec y) { return ew<EW_SCALE>(V(y), a, 0, V(x), nullptr); }
FS_API int fs_vec_scale_self(double a, fs_vec x) { return ew<EW_SCALE>(V(x), a, 0, V(x), nullptr); }
FS_API int fs_vec_add(fs_vec x, fs_vec y, fs_vec z) { return ew<EW_ADD>(V(z), 0, 0, V(x), V(y)); }
FS_API int fs_vec_subtract(fs_vec x, fs_vec y, fs_vec z) { return ew<EW_SUB>(V(z), 0, 0, V(x), V(y)); }
FS_API int fs_vec_multiply(fs_vec x, fs_vec y, fs_vec z) { return ew<EW_MUL>(V(z), 0, 0, V(x), V(y)); }
FS_API int fs_vec_divide(fs_vec x, fs_vec y, fs_vec z) { return ew<EW_DIV>(V(z), 0, 0, V(x), V(y)); }
FS_API int fs_vec_reciprocal(fs_vec x, fs_vec y) { return ew<EW_RECIP>(V(y), 0, 0, V(x), nullptr); }
FS_API int fs_vec_linear_sum(double a, fs_vec x, double b, fs_vec y, fs_vec z) {
	return ew<EW_LINSUM>(V(z), a, b, V(x), V(y));
}
FS_API int fs_vec_axpy(double a, fs_vec x, fs_vec y, fs_vec z) { return ew<EW_AXPY>(V(z), a, 0, V(x), V(y)); }
FS_API int fs_vec_axpby(double a, double b, fs_vec x, fs_vec z) { return ew<EW_AXPBY>(V(z), a, b, V(x), V(z)); }
FS_API int fs_vec_abs(fs_vec x, fs_vec y) { return ew<EW_ABS>(V(y), 0, 0, V(x), nullptr); }
FS_API int fs_vec_add_scalar(fs_vec x, double a, fs_vec y) { return ew<EW_ADDS>(V(y), a, 0, V(x), nullptr); }

FS_API int fs_vec_set_random(fs_vec h, uint64_t seed) {
	Vec *v = V(h);
	if (!ok_vec(v))
		return FS_ERR_BAD_HANDLE;
	if (v->n == 0)
		return FS_OK;
	int g = grid_for(v->ctx, v->n, 256, 4);
	if (v->dtype == FS_F64)
		rand_kernel<double><<<g, 256, 0, v->ctx->stream>>>(v->n, seed, (double *)v->d);
	else
		rand_kernel<float><<<g, 256, 0, v->ctx->stream>>>(v->n, seed, (float *)v->d);
	return check_launch(v->ctx, "set_random");
}

FS_API int fs_vec_dot(fs_vec x, fs_vec y, double *out) { return reduce<RD_DOT>(V(x), V(y), out); }
FS_API int fs_vec_l1norm(fs_vec x, double *out) { return reduce<RD_L1>(V(x), nullptr, out); }
FS_API int fs_vec_l2norm(fs_vec x, double *out) {
	FS_TRY(reduce<RD_DOT>(V(x), V(x), out));
	*out = std::sqrt(*out);
	return FS_OK;
}
FS_API int fs_vec_inf_norm(fs_vec x, double *out) { return reduce<RD_INF>(V(x), nullptr, out); }
FS_API int fs_vec_min(fs_vec x, double *out) { return reduce<RD_MIN>(V(x), nullptr, out); }
FS_API int fs_vec_max(fs_vec x, double *out) { return reduce<RD_MAX>(V(x), nullptr, out); }

#undef V

}  // extern "C"
