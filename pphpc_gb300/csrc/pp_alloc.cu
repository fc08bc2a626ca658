/*
 * pp_alloc.cu -- process-wide cache of the device buffers of worlds.
 *
 * A world allocates its state in about twenty buffers of up to a few GB
 * (12800^2: ~6 GB); cudaMalloc and cudaFree of that much take milliseconds,
 * as long as several iterations. Buffers a destroyed world frees are kept
 * per device and handed to a later allocation on that device that they fit
 * within a quarter of its size (best fit), so a process that runs job after
 * job (a service creating simulations, an end-to-end benchmark) allocates
 * from the driver once. The cache holds at most a quarter of the device's
 * memory (PP_CACHE_BYTES overrides the limit, 0 turns the cache off); an
 * allocation the driver refuses empties the device's cache and is retried;
 * pp_release_cached_memory empties it on request.
 */
#include <cstdlib>
#include <map>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/pphpc.h"
#include "pp_world.cuh"

namespace pp {

namespace {

struct DeviceCache {
	std::multimap<size_t, void *> blocks;   /* size -> buffer */
	size_t bytes = 0;
	size_t limit = 0;
	bool sized = false;
};

std::mutex g_mu;
std::map<int, DeviceCache> g_cache;

/* The cache limit of the current device (called with g_mu held). */
size_t limit_of(DeviceCache &c)
{
	if (!c.sized) {
		const char *env = getenv("PP_CACHE_BYTES");
		if (env) {
			c.limit = (size_t) strtoull(env, nullptr, 0);
		} else {
			size_t fr = 0, total = 0;
			if (cudaMemGetInfo(&fr, &total) != cudaSuccess) {
				cudaGetLastError();
				total = 0;
			}
			c.limit = total / 4;
		}
		c.sized = true;
	}
	return c.limit;
}

size_t release_locked(int device)
{
	size_t n = 0;
	for (auto &kv : g_cache) {
		if (device >= 0 && kv.first != device) continue;
		if (kv.second.blocks.empty()) continue;
		int cur = 0;
		cudaGetDevice(&cur);
		cudaSetDevice(kv.first);
		for (auto &b : kv.second.blocks) {
			cudaFree(b.second);
			n += b.first;
		}
		kv.second.blocks.clear();
		kv.second.bytes = 0;
		cudaSetDevice(cur);
	}
	return n;
}

} /* namespace */

cudaError_t cached_malloc(int device, size_t bytes, void **p, size_t *got)
{
	{
		std::lock_guard<std::mutex> lk(g_mu);
		DeviceCache &c = g_cache[device];
		auto it = c.blocks.lower_bound(bytes);
		if (it != c.blocks.end() && it->first - bytes <= bytes / 4) {
			*p = it->second;
			*got = it->first;
			c.bytes -= it->first;
			c.blocks.erase(it);
			return cudaSuccess;
		}
	}
	cudaError_t e = cudaMalloc(p, bytes);
	if (e == cudaErrorMemoryAllocation) {
		cudaGetLastError();
		std::lock_guard<std::mutex> lk(g_mu);
		if (release_locked(device) == 0) return e;
		e = cudaMalloc(p, bytes);
	}
	if (e == cudaSuccess) *got = bytes;
	return e;
}

void cached_free(int device, void *p, size_t bytes)
{
	if (!p) return;
	std::lock_guard<std::mutex> lk(g_mu);
	DeviceCache &c = g_cache[device];
	if (c.bytes + bytes <= limit_of(c)) {
		c.blocks.emplace(bytes, p);
		c.bytes += bytes;
	} else {
		cudaFree(p);
	}
}

} /* namespace pp */

extern "C" int pp_release_cached_memory(int device, uint64_t *released)
{
	size_t n;
	{
		std::lock_guard<std::mutex> lk(pp::g_mu);
		n = pp::release_locked(device);
	}
	if (released) *released = n;
	return PP_SUCCESS;
}
