// Host-side pieces of the persistent assembly kernel (batch.cu), shared by the
// batch API (batch.cu) and the serving loop (serve.cpp).  No device code here:
// the file is also compiled by the host compiler.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "fegpu_internal.h"

namespace fegpu {

// job kinds the kernel is compiled for: element type x form x DOFs per node
enum BatchCode {
  BC_H8_DIFF, BC_H20_DIFF, BC_T4_DIFF, BC_T10_DIFF, BC_Q4_DIFF,
  BC_H8_ELAST, BC_H20_ELAST, BC_T4_ELAST, BC_T10_ELAST,
  BC_Q4_DOT1, BC_Q4_DOT3, BC_H8_DOT1, BC_H8_DOT3,
  BC_COUNT
};

// Everything the kernel needs of one job (one matrix).
struct BatchJob {
  KArgs k;              // element stage (k.ke unused: the ring is g.ke)
  GArgs g;              // gather stage
  int code;             // BatchCode
  int form;             // F_DIFF_ISO, F_ELAST_ISO or F_DOT
  int etype;
  int ndn;
  int64_t elem_floats;  // floats of one element's block set (upper node pairs)
};

// One unit of work: an element tile (kind 0) or a range of the job's gather
// order (kind 1).  It may start once counters[dep[i]] >= target[i] (dep -1:
// none) and adds one to counters[done] when finished.
struct BatchItem {
  int job;
  int kind;
  int64_t b, e;
  int64_t chunk;
  int dep[2];
  int target[2];
  int done;
  int pad;
};

constexpr int kBatchThreads = 256;
constexpr int kBatchGatherNodes = 32;
// dynamic shared memory limit of the kernel (227 KB per CTA less its static part)
constexpr size_t kBatchMaxSmem = 227 * 1024 - 1024;
// coefficient kind of a dot job whose (matrix) coefficient is carried by cab/cdiag
constexpr int kCoefNone = -1;

int batch_code(int etype, int form, int ndn);
const char *batch_code_name(int code);

// Kernel arguments of one job.  Per-element / per-point coefficient values are
// copied (element order) into `coef`, allocated as needed, on stream s; `ring`
// replaces the dofmap's block ring when not null.  Builds the dofmap's gather
// plan on first use.
void make_batch_job(fegpu_matrix *K, int form, int code, int m, const fegpu_coef *cf, int te,
                    std::unique_ptr<DevBuf> &coef, float *ring, cudaStream_t s, BatchJob &out);

// Queue order of the items of a set of jobs, and the completion counters they
// use (returned).  Per job the stages run E0, E1, G0, E2, G1, ... (E: element
// blocks of a chunk, G: gather of the nodes completed by that chunk); E(c)
// waits for E(c-1) and for the last gather that reads its ring slot's previous
// chunk, G(c) for E(c) and G(c-1), so a chunk's element tiles overlap the
// previous chunk's gather.  Jobs
// pass through a window (one stage of each per round) holding the jobs whose
// live ring chunks fit in `live_budget` bytes (at least two jobs).
// ranges (optional): per job the chunks [c0, c1) to run (a slice of the job,
// whose earlier chunks ran in launches before this one on the same stream).
struct ChunkRange {
  int64_t c0, c1;
};
int build_batch_items(const std::vector<BatchJob> &jobs,
                      const std::vector<const fegpu_dofmap *> &dms, size_t live_budget,
                      std::vector<BatchItem> &items,
                      const std::vector<ChunkRange> *ranges = nullptr);

// Dynamic shared memory the kernel needs for these jobs.
size_t batch_smem_bytes(const std::vector<BatchJob> &jobs,
                        const std::vector<const fegpu_dofmap *> &dms);

// Persistent grid: resident CTAs per SM x SMs x share (0 < share <= 1).
int batch_grid(int num_sms, size_t smem, int nitems, double share);

// Launch of the persistent kernel (status: 0 ok, 1 a wait ran out of time);
// withheld >= 0 withholds the completions of that counter (the failure path's
// test: the items waiting on it run out of time).
void launch_batch_kernel(int grid, size_t smem, cudaStream_t s, const BatchJob *jobs,
                         const BatchItem *items, int nitems, int *next, int *counters,
                         int *status, double wait_s, int withheld = -1);

}  // namespace fegpu
