// Copy / compute timeline probe: a CUPTI activity tracer loaded into a process
// through CUDA_INJECTION64_PATH (the CUDA driver calls InitializeInjection at
// initialisation).  It records every kernel (concurrent-kernel activity) and
// every memcpy with their GPU start/end timestamps, stream and bytes, and writes
// them as CSV to $OVERLAP_TRACE_OUT when the process exits.  A host program
// that also dlopen()s this library can call overlap_trace_mark(label) to put a
// timestamped marker line between the calls it wants summarised
// (overlap_summary.py computes busy time and overlap per window).
//
// Build (on the GPU machine):
//   nvcc -O2 -shared -Xcompiler -fPIC tiled-mm_gb300/peaks/overlap_trace.cpp \
//        -o tiled-mm_gb300/peaks/_build/liboverlap_trace.so -lcupti -Xlinker -rpath=/usr/local/cuda/lib64
#include <cupti.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace {

std::mutex g_mu;
std::vector<std::string> g_lines;
bool g_started = false;

const char* copy_kind(uint8_t k) {
  switch (k) {
    case CUPTI_ACTIVITY_MEMCPY_KIND_HTOD: return "H2D";
    case CUPTI_ACTIVITY_MEMCPY_KIND_DTOH: return "D2H";
    case CUPTI_ACTIVITY_MEMCPY_KIND_DTOD: return "D2D";
    case CUPTI_ACTIVITY_MEMCPY_KIND_HTOH: return "H2H";
    default: return "other";
  }
}

void CUPTIAPI buffer_requested(uint8_t** buffer, size_t* size, size_t* max_records) {
  constexpr size_t BYTES = 8u << 20;
  *buffer = (uint8_t*)aligned_alloc(8, BYTES);
  *size = *buffer ? BYTES : 0;
  *max_records = 0;
}

void CUPTIAPI buffer_completed(CUcontext, uint32_t, uint8_t* buffer, size_t, size_t valid) {
  CUpti_Activity* rec = nullptr;
  std::vector<std::string> out;
  while (cuptiActivityGetNextRecord(buffer, valid, &rec) == CUPTI_SUCCESS) {
    char line[512];
    if (rec->kind == CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL || rec->kind == CUPTI_ACTIVITY_KIND_KERNEL) {
      const CUpti_ActivityKernel10* k = (const CUpti_ActivityKernel10*)rec;
      std::string name = k->name ? k->name : "?";
      for (char& c : name)
        if (c == ',') c = ';';
      snprintf(line, sizeof line, "kernel,%s,%u,%llu,%llu,0", name.substr(0, 200).c_str(), k->streamId,
               (unsigned long long)k->start, (unsigned long long)k->end);
      out.emplace_back(line);
    } else if (rec->kind == CUPTI_ACTIVITY_KIND_MEMCPY) {
      const CUpti_ActivityMemcpy6* m = (const CUpti_ActivityMemcpy6*)rec;
      snprintf(line, sizeof line, "memcpy,%s,%u,%llu,%llu,%llu", copy_kind(m->copyKind), m->streamId,
               (unsigned long long)m->start, (unsigned long long)m->end, (unsigned long long)m->bytes);
      out.emplace_back(line);
    }
  }
  free(buffer);
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto& l : out) g_lines.push_back(std::move(l));
}

void write_out() {
  cuptiActivityFlushAll(1);
  const char* path = getenv("OVERLAP_TRACE_OUT");
  if (!path) return;
  std::lock_guard<std::mutex> lock(g_mu);
  FILE* f = fopen(path, "w");
  if (!f) return;
  fprintf(f, "what,name,stream,start_ns,end_ns,bytes\n");
  for (const auto& l : g_lines) fprintf(f, "%s\n", l.c_str());
  fclose(f);
}

}  // namespace

extern "C" int InitializeInjection(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_started) return 1;
  g_started = true;
  if (cuptiActivityRegisterCallbacks(buffer_requested, buffer_completed) != CUPTI_SUCCESS) return 0;
  cuptiActivityEnable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL);
  cuptiActivityEnable(CUPTI_ACTIVITY_KIND_MEMCPY);
  atexit(write_out);
  return 1;
}

// a marker between the calls to summarise (GPU timestamp domain of the activity records)
extern "C" void overlap_trace_mark(const char* label) {
  uint64_t t = 0;
  cuptiGetTimestamp(&t);
  char line[256];
  snprintf(line, sizeof line, "mark,%s,0,%llu,%llu,0", label ? label : "", (unsigned long long)t,
           (unsigned long long)t);
  std::lock_guard<std::mutex> lock(g_mu);
  g_lines.emplace_back(line);
}
