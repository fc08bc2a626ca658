/*
 * pp_cpu_kernels.cpp -- the reference's CPU kernels, compiled unmodified.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/ref/build_ref.py). This translation
 * unit is ocl_compat.hpp followed by the reference's own kernel sources in
 * the order its host concatenates them (pp_cpu.c:965-967: RNG source, then
 * pp_common.cl, then pp_cpu.cl), included from the reference tree by the
 * build recipe (-I <reference>/opencl/pp), plus one host entry per kernel
 * that runs one work item.
 */
#include "ocl_compat.hpp"

namespace ocl {
typedef uint_t uint;
#include "pp_common.cl"
#include "pp_cpu.cl"
} /* namespace ocl */

/* One work item (gid of gws) of each kernel; the host loop sets the
 * work-item identity of the calling thread first. */
extern "C" {

void ppr_kernel_init(void *agents, void *cells, void *stats, void *seeds,
	unsigned long gid, unsigned long gws)
{
	ocl::tl_gid = gid;
	ocl::tl_gws = gws;
	ocl::init((ocl::PPCAgentOcl *) agents, (ocl::PPCCellOcl *) cells,
		(ocl::PPStatisticsOcl *) stats, (ocl::clo_statetype *) seeds);
}

void ppr_kernel_step1(void *agents, void *cells, void *seeds, unsigned turn,
	unsigned long gid, unsigned long gws)
{
	ocl::tl_gid = gid;
	ocl::tl_gws = gws;
	ocl::step1((ocl::PPCAgentOcl *) agents, (ocl::PPCCellOcl *) cells,
		(ocl::clo_statetype *) seeds, turn);
}

void ppr_kernel_step2(void *agents, void *cells, void *seeds, void *stats,
	unsigned iter, unsigned turn, unsigned long gid, unsigned long gws)
{
	ocl::tl_gid = gid;
	ocl::tl_gws = gws;
	ocl::step2((ocl::PPCAgentOcl *) agents, (ocl::PPCCellOcl *) cells,
		(ocl::clo_statetype *) seeds, (ocl::PPStatisticsOcl *) stats, iter, turn);
}

/* Sizes the host loop allocates by (pp_cpu.c:470-480: 8 bytes per cell and
 * per agent slot here; the reference sizes its agent buffer at 16 bytes a
 * slot, of which its kernel uses 8). */
unsigned long ppr_sizeof_agent(void) { return sizeof(ocl::PPCAgentOcl); }
unsigned long ppr_sizeof_cell(void) { return sizeof(ocl::PPCCellOcl); }
unsigned long ppr_sizeof_stats(void) { return sizeof(ocl::PPStatisticsOcl); }

}
