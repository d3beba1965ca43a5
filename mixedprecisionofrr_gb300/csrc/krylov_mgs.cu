// Orthogonal Arnoldi step with modified Gram-Schmidt (and optional reorthogonalisation), the FP64
// comparison path arnoldi_mgs_eig.m:57-112.  For new column w = V(:, i):
//   for j = 0..i-1:  r = dot(w, v_j) (pc, rounded to po);  w = po(pc(w) - pc(r) pc(v_j))   [twice with reorth]
//   t = norm2(w) (pc, rounded to po);  t < select_tol -> breakdown;  w = po(pc(w) / pc(t))
// Every dot product is a grid reduction (per-CTA partial sums, the last CTA to finish adds them in a
// fixed order, so results are deterministic); the MGS order makes the j loop sequential.  A device
// stop word records a breakdown and turns the rest of the cycle into no-ops without a host sync.
#include "ofrr_internal.cuh"

namespace ofrr {

constexpr int MG_T = 256;
constexpr int MG_GRID = 152 * 2;

// partial[blockIdx] = sum over this CTA's rows of pc(x) pc(y) (y == nullptr: pc(x)^2); the last CTA
// reduces the partials in order and stores out = po(total) (sqrt first when y == nullptr), plus the
// breakdown test for norms.
template <class TO, class TC>
__global__ void __launch_bounds__(MG_T) k_mgs_reduce(int64_t n, const TO* __restrict__ x, const TO* __restrict__ y,
                                                     TC* __restrict__ partial, unsigned int* __restrict__ counter,
                                                     TO* __restrict__ out, int step, double stol,
                                                     int* __restrict__ stop) {
  __shared__ TC red[MG_T / 32];
  __shared__ bool last;
  if (*stop >= 0) return;
  TC s = TC(0);
  for (int64_t i = blockIdx.x * (int64_t)MG_T + threadIdx.x; i < n; i += (int64_t)gridDim.x * MG_T) {
    const TC a = to_c<TC, TO>(x[i]);
    s += a * (y ? to_c<TC, TO>(y[i]) : a);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    TC b = TC(0);
    for (int w = 0; w < MG_T / 32; ++w) b += red[w];
    partial[blockIdx.x] = b;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const volatile TC* vp = partial;
  TC tot = TC(0);
  for (unsigned int b = 0; b < gridDim.x; ++b) tot += vp[b];
  *counter = 0;  // self-resetting for the next reduction
  if (y == nullptr) {
    const TO t = from_c<TO, TC>(sqrt(tot));
    *out = t;
    if (absd(t) < stol) *stop = step;  // breakdown: invariant subspace
  } else {
    *out = from_c<TO, TC>(tot);
  }
}

// x = po(pc(x) - pc(r) pc(v))  (v != nullptr), or x = po(pc(x) / pc(r)) (v == nullptr)
template <class TO, class TC>
__global__ void __launch_bounds__(MG_T) k_mgs_update(int64_t n, TO* __restrict__ x, const TO* __restrict__ v,
                                                     const TO* __restrict__ r, const int* __restrict__ stop) {
  if (*stop >= 0) return;
  const TC rc = to_c<TC, TO>(*r);
  for (int64_t i = blockIdx.x * (int64_t)MG_T + threadIdx.x; i < n; i += (int64_t)gridDim.x * MG_T) {
    const TC a = to_c<TC, TO>(x[i]);
    x[i] = v ? from_c<TO, TC>(a - rc * to_c<TC, TO>(v[i])) : from_c<TO, TC>(a / rc);
  }
}

// Orthogonalise column i of V (n x nb, ld ldv) against columns 0..i-1 and normalise it.  scratch:
// MG_GRID partials (TC) + a counter (zero on entry, left zero) + one TO word for r / t.
template <class TO, class TC>
static int mgs_step_t(ofrr_ctx* ctx, int64_t n, int i, TO* V, int64_t ldv, bool reorth, double stol, int* stop,
                      void* scratch) {
  TC* partial = (TC*)scratch;
  unsigned int* counter = (unsigned int*)((char*)scratch + 8 * MG_GRID);
  TO* rw = (TO*)((char*)scratch + 8 * MG_GRID + 16);
  const int grid = grid_for(n, MG_T, MG_GRID);
  TO* w = V + (int64_t)i * ldv;
  for (int j = 0; j < i; ++j) {
    const TO* vj = V + (int64_t)j * ldv;
    for (int pass = 0; pass < (reorth ? 2 : 1); ++pass) {
      k_mgs_reduce<TO, TC><<<grid, MG_T, 0, ctx->stream>>>(n, w, vj, partial, counter, rw, i, stol, stop);
      OFRR_LAUNCHED(ctx, "k_mgs_reduce");
      k_mgs_update<TO, TC><<<grid, MG_T, 0, ctx->stream>>>(n, w, vj, rw, stop);
      OFRR_LAUNCHED(ctx, "k_mgs_update");
    }
  }
  k_mgs_reduce<TO, TC><<<grid, MG_T, 0, ctx->stream>>>(n, w, nullptr, partial, counter, rw, i, stol, stop);
  OFRR_LAUNCHED(ctx, "k_mgs_reduce");
  k_mgs_update<TO, TC><<<grid, MG_T, 0, ctx->stream>>>(n, w, nullptr, rw, stop);
  OFRR_LAUNCHED(ctx, "k_mgs_update");
  return OFRR_SUCCESS;
}

size_t mgs_scratch_bytes() { return 8 * MG_GRID + 16 + 16; }

int mgs_step(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t n, int i, void* V, int64_t ldv, bool reorth,
             double stol, int* stop, void* scratch) {
  OFRR_DISPATCH_STORAGE(po, TO, OFRR_DISPATCH_COMPUTE(pc, TC, {
    OFRR_TRY((mgs_step_t<TO, TC>(ctx, n, i, (TO*)V, ldv, reorth, stol, stop, scratch)));
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr
