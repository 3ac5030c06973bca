// Internal state of a tmm_context (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tmm_c_api.h"
#include "tmm_batched.h"

namespace tmm {

// A device allocation that only grows (src/Tiled-MM/device_vector.hpp:93-107:
// capacity 1.2x the requested size when it has to grow).
struct GrowBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;     // requested size
  size_t capacity = 0;  // allocated size
  cudaError_t reserve(size_t want);
  void release();
};

// One device-resident A or B tile (raw FP64/FP32/complex, or Ozaki digit planes).
struct Slot {
  char* ptr = nullptr;
  cudaEvent_t ready = nullptr;     // recorded when the tile's data is in place
  cudaEvent_t last_use = nullptr;  // recorded after the last kernel that read it
  int64_t key = -1;
  uint64_t stamp = 0;
  bool used = false;               // last_use has been recorded
};

struct TileCache {
  std::vector<Slot> slots;
  std::unordered_map<int64_t, int> index;
  uint64_t clock = 0;
  void invalidate() {
    index.clear();
    for (auto& s : slots) { s.key = -1; s.used = false; }
  }
  // slot holding key, or -1
  int find(int64_t key) {
    auto it = index.find(key);
    return it == index.end() ? -1 : it->second;
  }
  // least recently used slot (free slots first)
  int victim() {
    int best = -1;
    for (int i = 0; i < (int)slots.size(); ++i) {
      if (slots[i].key < 0) return i;
      if (best < 0 || slots[i].stamp < slots[best].stamp) best = i;
    }
    return best;
  }
};

struct CSlot {
  char* ptr = nullptr;
  cudaEvent_t done = nullptr;  // the slot's previous tile has left for the host
  bool used = false;
};

struct OzakiState;  // defined with the Ozaki engine

}  // namespace tmm

struct tmm_context {
  int dtype = TMM_DOUBLE;
  int device = 0;
  int n_streams = 2;
  int max_tile_m = 5000, max_tile_n = 5000, max_tile_k = 5000;
  int cur_tile_m = 0, cur_tile_n = 0, cur_tile_k = 0;  // tile sizes of the last call (0 = none yet)
  int path = TMM_PATH_NATIVE;
  int ozaki_slices = 0;
  int tile_policy = TMM_TILE_POLICY_REFERENCE;
  size_t memory_limit = 0;
  // TMM_DIRECT_HOST=1 and the GPU reads and writes ordinary (pageable) host memory through the
  // host page tables: tiles of unregistered host buffers are copied by kernel
  bool direct_host = false;

  std::vector<cudaStream_t> streams;  // compute streams
  cudaStream_t h2d = nullptr;         // host -> device copies
  cudaStream_t prep = nullptr;        // tile preparation kernels (Ozaki split)
  cudaStream_t d2h = nullptr;         // result stream (src/Tiled-MM/gpu_context.hpp:39)

  tmm::GrowBuffer pool_a, pool_b, pool_c, full_c, staging, scratch;
  tmm::GrowBuffer oz_work;  // [256-byte error word block][per-stream FP64 workspaces of the tcgen05 engine]
  int oz_engine = 0;

  // batched path: packed operands, device problem records + work list, and the
  // CUDA graph captured for the last batch layout
  tmm::GrowBuffer batch_arena, batch_meta;
  std::vector<unsigned char> batch_key;
  cudaGraphExec_t batch_exec = nullptr;
  cudaStream_t batch_aux = nullptr;  // second stream: FP32 items beside the FP64 items
  cudaEvent_t batch_fork = nullptr, batch_join = nullptr;
  tmm::TileCache cache_a, cache_b;
  std::vector<tmm::CSlot> cslots;  // 2 per stream
  std::vector<cudaEvent_t> staging_free;
  size_t full_c_elems = 0;

  tmm::OzakiState* oz = nullptr;

  // float and complex on the Ozaki engine: embedding, digit planes and real product, per stream slot
  std::vector<tmm::GrowBuffer> cz_scratch;

  // batched FP64 problems on the Ozaki path: digit planes per branch stream, the branch
  // streams and their join events
  tmm::GrowBuffer batch_oz_scratch;
  std::vector<cudaStream_t> oz_branches;
  std::vector<cudaEvent_t> oz_branch_done;
  cudaEvent_t oz_fork = nullptr;

  // optional timing of the engine kernels (tmm_set_kernel_timing): event pairs recorded
  // on the launching stream around each launch, summed by tmm_get_kernel_time

  bool ktime = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kt_pending, kt_free;
  double kt_seconds = 0.0;
  uint64_t kt_launches = 0;
  // origin event recorded when timing is switched on; each timed launch's (start, end)
  // relative to it, for the union of busy time over launches on several streams
  cudaEvent_t kt_origin = nullptr;
  std::vector<std::pair<double, double>> kt_intervals;

  tmm_stats stats{};
  std::string last_error;
  // FP32 tensor-core engine: per stream slot (the compute streams, then one for other
  // streams), a 256-byte error-word header and the bf16 planes of the tile operands
  std::vector<tmm::GrowBuffer> f32_scratch;
  // batched FP32 problems on that engine: [error word][planes][grouped launch records], and the
  // stream they run on beside the batch stream
  tmm::GrowBuffer batch_f32_scratch;
  cudaStream_t batch_f32_stream = nullptr;
  cudaEvent_t batch_f32_fork = nullptr, batch_f32_join = nullptr;
  // lanes of the batch's many small launches and copies (the FP32 problems' splits, the
  // copies back of the problems outside the Ozaki pipeline): forked from and joined into the
  // stream that would otherwise run them one after another
  std::vector<cudaStream_t> batch_lanes;
  std::vector<cudaEvent_t> batch_lane_events;  // [0]: fork, [1 + i]: lane i done
  bool f32_simt = false;  // TMM_F32_KERNEL=simt: the FFMA tile kernel instead

  // the size class of the last autotuned call (tmm_get_autotune_report)
  tmm::TuneProblem last_tune{};
  bool has_tune = false;
};
