/*
 * pp_noalloc.cu -- a radix sort entry point that allocates no device memory.
 *
 * pp_radix_sort_host allocates its buffers and its scratch (look-back
 * words, digit histograms, counters) with cudaMalloc on every call. Some
 * callers cannot do that: an application whose memory is owned by its own
 * pooling allocator (a raw cudaMalloc would bypass the pool's budget and
 * fragment it), or a loop with a latency budget, where cudaMalloc and
 * cudaFree can synchronise the whole device. pp_radix_sort_noalloc serves
 * them: the caller passes device buffers for the data, and the sort's
 * scratch lives in the file-scope array below, sized for at most
 * PP_NOALLOC_SORT_MAX_N pairs. Every GPU that loads this library holds the
 * array (about 2 MB) until the process exits.
 */
#include <mutex>

#include "pp_kernels.cuh"

namespace pp {

int occupancy_sort(int dbits);
int cuda_status(cudaError_t e);

namespace {

constexpr uint32_t MAX_N = PP_NOALLOC_SORT_MAX_N;
constexpr size_t MAX_TILES = (MAX_N + SORT_TILE - 1) / SORT_TILE + 1;
constexpr size_t LB_BYTES = MAX_TILES * 256 * sizeof(uint64_t);
constexpr size_t HIST_OFF = LB_BYTES;
constexpr size_t HIST_BYTES = 8 * 256 * sizeof(uint32_t);
constexpr size_t CTR_OFF = HIST_OFF + HIST_BYTES;
constexpr size_t N_OFF = CTR_OFF + ((sizeof(WorldCounters) + 255) / 256) * 256;
constexpr size_t SCRATCH_BYTES = N_OFF + 256;

/* Shared by every call on a device: look-back words, then the digit
 * histograms, the counters and the element count. */
static __device__ __align__(256) unsigned char g_sort_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void *g_addr[MAX_DEVICES];
int g_sms[MAX_DEVICES];

/* Device address of the scratch array on the current device. In host code
 * the symbol itself is only a host-side stand-in, so the address must come
 * from cudaGetSymbolAddress, once per device, with that device current. */
cudaError_t scratch_on_current_device(void **addr, int *sms)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> lock(g_mu);
	if (!g_addr[dev]) {
		void *p = nullptr;
		e = cudaGetSymbolAddress(&p, g_sort_scratch);
		if (e != cudaSuccess) return e;
		int n = 0;
		e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
		if (e != cudaSuccess) return e;
		g_addr[dev] = p;
		g_sms[dev] = n;
	}
	*addr = g_addr[dev];
	*sms = g_sms[dev];
	return cudaSuccess;
}

} /* namespace */
} /* namespace pp */

using namespace pp;

extern "C" int pp_radix_sort_noalloc(uint32_t n, uint32_t *keys,
	uint32_t *vals, uint32_t *keys_out, uint32_t *vals_out,
	uint32_t key_bits, uint32_t digit_bits, void *stream)
{
	if (n > MAX_N) return PP_INVALID_ARGS;
	if (key_bits == 0 || key_bits > 32) return PP_INVALID_ARGS;
	if (n && (!keys || !vals || !keys_out || !vals_out)) return PP_INVALID_ARGS;
	uint32_t d = digit_bits;
	if (d == 0) {
		uint32_t passes = (key_bits + 7) / 8;
		d = (key_bits + passes - 1) / passes;
		if (d < 5) d = 5;
	}
	if (d < 5 || d > 8) return PP_INVALID_ARGS;
	const uint32_t passes = (key_bits + d - 1) / d;
	cudaStream_t s = (cudaStream_t) stream;
	if (n == 0) return PP_SUCCESS;

	void *base = nullptr;
	int sms = 0;
	cudaError_t e = scratch_on_current_device(&base, &sms);
	if (e != cudaSuccess) return cuda_status(e);
	unsigned char *sc = (unsigned char *) base;
	uint64_t *lb = (uint64_t *) sc;
	uint32_t *hist = (uint32_t *) (sc + HIST_OFF);
	WorldCounters *ctr = (WorldCounters *) (sc + CTR_OFF);
	uint32_t *n_dev = (uint32_t *) (sc + N_OFF);

	/* The array keeps the previous call's contents: clear the look-back
	 * words this sort will use, the histograms and the counters. */
	const size_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
	e = cudaMemsetAsync(lb, 0, tiles * 256 * sizeof(uint64_t), s);
	if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, HIST_BYTES, s);
	if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(WorldCounters), s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(n_dev, &n, sizeof(n), cudaMemcpyHostToDevice, s);
	if (e == cudaSuccess)
		e = launch_radix_hist(keys, n_dev, hist, d, passes, sms * 4, s);
	int occ = occupancy_sort((int) d);
	uint32_t *ki = keys, *vi = vals, *ko = keys_out, *vo = vals_out;
	for (uint32_t p = 0; p < passes && e == cudaSuccess; p++) {
		e = launch_radix_pass(ki, vi, ko, vo, hist + p * 256, lb, ctr, n_dev,
			p, p * d, d, sms * (occ > 0 ? occ : 1), s);
		std::swap(ki, ko);
		std::swap(vi, vo);
	}
	/* After an even number of passes the result is in the input buffers. */
	if (e == cudaSuccess && ki != keys_out) {
		e = cudaMemcpyAsync(keys_out, ki, (size_t) n * 4, cudaMemcpyDeviceToDevice, s);
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(vals_out, vi, (size_t) n * 4, cudaMemcpyDeviceToDevice, s);
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return cuda_status(e);
	uint32_t err = 0;
	e = cudaMemcpy(&err, &ctr->err, sizeof(err), cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) return cuda_status(e);
	return (err & ERRF_TIMEOUT) ? PP_ERR_TIMEOUT : PP_SUCCESS;
}
