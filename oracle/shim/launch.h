// Launch loop for a generated kernel compiled against cuda_runtime.h above.
#pragma once

#include <algorithm>
#include <memory>
#include <thread>
#include <vector>

namespace vdx_shim {
thread_local uint3 tid;
uint3 bid;
dim3 bdim;
dim3 gdim;
std::barrier<>* bar;
thread_local int lin;
Warp* warps;

template <class F>
void run_grid(dim3 grid, dim3 block, F&& body) {
  gdim = grid;
  bdim = block;
  const int nthreads = int(block.x * block.y * block.z);
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        bid = uint3{bx, by, bz};
        std::barrier<> b(nthreads);
        bar = &b;
        const int nwarps = (nthreads + 31) / 32;
        std::vector<Warp> ws(nwarps);
        std::vector<std::unique_ptr<std::barrier<>>> wbars;
        for (int w = 0; w < nwarps; ++w) {
          wbars.emplace_back(new std::barrier<>(std::min(32, nthreads - 32 * w)));
          ws[w].bar = wbars.back().get();
        }
        warps = ws.data();
        std::vector<std::thread> ts;
        ts.reserve(nthreads);
        for (int t = 0; t < nthreads; ++t)
          ts.emplace_back([&, t] {
            tid = uint3{unsigned(t % block.x), unsigned((t / block.x) % block.y), unsigned(t / (block.x * block.y))};
            lin = t;
            body();
          });
        for (auto& th : ts) th.join();
      }
}
}  // namespace vdx_shim
