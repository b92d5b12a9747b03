// Pinned host memory on transparent huge pages, for the host-buffer entry
// point (tokura_zgeev_batched_host) and callers that stage their own copies.
//
// cudaHostAlloc pins base pages (4 KB or 64 KB). Where device DMA to host
// memory goes through an IOMMU, the device then needs one address translation
// per base page, and those translations are not kept while the copy engines
// are idle: on the GB300 machines measured here a 2 GiB copy from cudaHostAlloc
// memory ran at 211 GB/s back to back, 189 GB/s after 3 s idle and 110-134 GB/s
// after 5 s, while the same copy from memory mapped with MADV_HUGEPAGE and
// then registered (cudaHostRegister) ran at 210-211 GB/s after every idle
// period. tokuraHostAlloc maps anonymous memory aligned to the huge-page size,
// asks for huge pages, and registers it with CUDA (which faults the pages in).
// Buffers smaller than one huge page get base pages and are only registered.
#include <sys/mman.h>
#include <unistd.h>

#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "../../include/tokura_blas_ext.h"

namespace {

std::mutex g_mu;
std::map<void*, size_t> g_maps;  // start -> length of each live mapping

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Size of a transparent huge page (the PMD size): the kernel reports it, or
// it is derived from the base page (a page-table page holds page/8 entries).
size_t huge_page_bytes() {
  size_t hp = 0;
  if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
    if (std::fscanf(f, "%zu", &hp) != 1) hp = 0;
    std::fclose(f);
  }
  if (hp == 0) {
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    hp = page * (page / 8);
  }
  return hp;
}

}  // namespace

extern "C" TOKURA_API int tokuraHostAlloc(void** ptr, size_t bytes) {
  if (ptr == nullptr) return -1;
  *ptr = nullptr;
  if (bytes == 0) return -2;
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  const size_t hp = huge_page_bytes();
  if (bytes > ~(size_t)0 - 2 * (hp > page ? hp : page)) return 2;  // the rounded mapping would overflow
  const size_t len = round_up(bytes, page);
  const bool huge = hp > page && len >= hp;
  // Map with room to align the start to a huge page, then trim both ends.
  const size_t map_len = huge ? len + hp : len;
  void* base = mmap(nullptr, map_len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (base == MAP_FAILED) return 2;
  char* start = static_cast<char*>(base);
  if (huge) {
    start = reinterpret_cast<char*>(round_up(reinterpret_cast<size_t>(base), hp));
    const size_t head = (size_t)(start - static_cast<char*>(base));
    if (head > 0) munmap(base, head);
    const size_t tail = map_len - head - len;
    if (tail > 0) munmap(start + len, tail);
    madvise(start, len, MADV_HUGEPAGE);  // advisory: base pages if the kernel declines
  }
  if (cudaHostRegister(start, len, cudaHostRegisterDefault) != cudaSuccess) {
    munmap(start, len);
    return 1;
  }
  {
    std::lock_guard<std::mutex> lock(g_mu);
    g_maps[start] = len;
  }
  *ptr = start;
  return 0;
}

extern "C" TOKURA_API int tokuraHostFree(void* ptr) {
  if (ptr == nullptr) return 0;
  size_t len;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_maps.find(ptr);
    if (it == g_maps.end()) return -1;
    len = it->second;
    g_maps.erase(it);
  }
  const cudaError_t err = cudaHostUnregister(ptr);
  munmap(ptr, len);
  return err == cudaSuccess ? 0 : 1;
}
