// Host-side check of the HBM arena's bookkeeping: many threads allocate,
// hand blocks to each other and free them; no two live blocks may overlap,
// every block lies inside the slab with the arena's alignment, and the used
// byte count returns to zero; regions (blocks whose interior another
// allocator hands out) return to the arena with their last reference.  The
// slab is a fake address range the arena never dereferences.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "../vedas_gb300/csrc/vg_ctx.h"

struct Block {
  uintptr_t a;
  size_t n;
};

int main(int argc, char** argv) {
  const int threads = argc > 1 ? std::atoi(argv[1]) : 16;
  const int ops = argc > 2 ? std::atoi(argv[2]) : 100000;
  const size_t cap = size_t{64} << 30;
  const uintptr_t base = uintptr_t{1} << 44;
  vg::Arena ar;
  ar.init_at(reinterpret_cast<void*>(base), cap);
  std::mutex hand_mu;
  std::vector<void*> handed;   // blocks passed between threads
  std::vector<std::vector<Block>> live(threads);
  std::vector<int> failures(threads, 0);
  auto worker = [&](int t) {
    std::mt19937_64 rng(1234 + t);
    std::vector<Block>& mine = live[t];
    for (int i = 0; i < ops; ++i) {
      const unsigned r = rng() % 100;
      if (r < 50 || mine.empty()) {
        size_t n;
        const unsigned k = rng() % 100;
        if (k < 70) n = 1 + rng() % 4096;
        else if (k < 95) n = 4096 + rng() % (1u << 20);
        else n = (1u << 20) + rng() % (16u << 20);
        void* p = ar.try_alloc(n);
        if (!p) {
          failures[t]++;
          continue;
        }
        mine.push_back({reinterpret_cast<uintptr_t>(p), n});
      } else if (r < 85) {  // free one of its own
        const size_t j = rng() % mine.size();
        ar.free(reinterpret_cast<void*>(mine[j].a));
        mine[j] = mine.back();
        mine.pop_back();
      } else if (r < 95) {
        const size_t j = rng() % mine.size();
        std::lock_guard<std::mutex> lk(hand_mu);
        handed.push_back(reinterpret_cast<void*>(mine[j].a));
        mine[j] = mine.back();
        mine.pop_back();
      } else {
        void* p = nullptr;
        {
          std::lock_guard<std::mutex> lk(hand_mu);
          if (!handed.empty()) {
            p = handed.back();
            handed.pop_back();
          }
        }
        if (p) ar.free(p);
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < threads; ++t) th.emplace_back(worker, t);
  for (auto& x : th) x.join();
  // every live block (still held or handed over but not freed) is disjoint
  std::vector<Block> all;
  for (auto& v : live) all.insert(all.end(), v.begin(), v.end());
  int bad = 0;
  for (const Block& b : all) {
    if (b.a < base || b.a + b.n > base + cap || (b.a - base) % vg::Arena::kAlign) ++bad;
  }
  std::sort(all.begin(), all.end(), [](const Block& x, const Block& y) { return x.a < y.a; });
  for (size_t i = 1; i < all.size(); ++i)
    if (all[i - 1].a + all[i - 1].n > all[i].a) ++bad;
  for (auto& v : live)
    for (const Block& b : v) ar.free(reinterpret_cast<void*>(b.a));
  for (void* p : handed) ar.free(p);
  // a large block shrinks and its tail is reusable
  void* big = ar.alloc(size_t{1} << 30);
  ar.shrink(big, size_t{1} << 20);
  const size_t used_after_shrink = ar.used();
  ar.free(big);
  const bool oom_ok = ar.try_alloc(cap + 1) == nullptr;
  // an allocation that does not fit first lets deferred releases run (the
  // reclaim hook), then retries: here the hook frees a block that fills the slab
  static vg::Arena* g_ar = nullptr;
  static void* g_held = nullptr;
  g_ar = &ar;
  const size_t lf = ar.largest_free();
  g_held = ar.alloc(lf);
  const bool setup_ok = ar.largest_free() < lf;   // a second request of lf bytes cannot fit now
  vg::set_arena_reclaim([] {
    if (g_held) g_ar->free(g_held);
    g_held = nullptr;
  });
  bool reclaim_ok = false;
  try {
    void* p = ar.alloc(lf);   // fits only after the hook ran
    reclaim_ok = setup_ok && p != nullptr && g_held == nullptr;
    ar.free(p);
  } catch (...) {
  }
  vg::set_arena_reclaim(nullptr);
  const bool peak_ok = ar.peak() >= lf;
  // regions: interior blocks handed out from a region are freed by many
  // threads (as relations are, on the host workers) while the opener closes
  // it; the region's block returns to the arena with the last reference, and
  // a block carved from the same bytes afterwards is freed normally
  bool region_ok = true;
  {
    const size_t used0 = ar.used();
    for (int round = 0; round < 20 && region_ok; ++round) {
      vg::Arena::Region* r = ar.region_open(size_t{256} << 20);
      if (!r) {
        region_ok = false;
        break;
      }
      const int per = 2000;
      std::vector<void*> interior;
      for (int i = 0; i < threads * per; ++i) interior.push_back(r->begin + size_t(i) * 4096);
      ar.region_adopt(r, static_cast<int64_t>(interior.size()));
      std::vector<std::thread> fr;
      for (int t = 0; t < threads; ++t)
        fr.emplace_back([&, t] {
          for (int i = t; i < static_cast<int>(interior.size()); i += threads) ar.free(interior[i]);
        });
      if (round & 1) ar.region_close(r);            // closed while its blocks are being freed
      for (auto& x : fr) x.join();
      if (!(round & 1)) ar.region_close(r);         // closed after every block was freed
      if (ar.used() != used0) region_ok = false;
      void* again = ar.alloc(size_t{64} << 20);     // reuses the region's bytes; a plain free
      ar.free(again);
      if (ar.used() != used0) region_ok = false;
    }
  }
  int fails = 0;
  for (int f : failures) fails += f;
  std::printf("blocks=%zu overlaps_or_out_of_range=%d used_end=%zu shrink_used=%zu oom_ok=%d alloc_failures=%d "
              "reclaim_ok=%d peak_ok=%d region_ok=%d\n",
              all.size(), bad, ar.used(), used_after_shrink, oom_ok ? 1 : 0, fails, reclaim_ok ? 1 : 0,
              peak_ok ? 1 : 0, region_ok ? 1 : 0);
  const bool ok = bad == 0 && ar.used() == 0 && used_after_shrink == (size_t{1} << 20) && oom_ok && fails == 0 &&
                  reclaim_ok && peak_ok && region_ok;
  return ok ? 0 : 1;
}
