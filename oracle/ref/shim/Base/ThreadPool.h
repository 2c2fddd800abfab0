/*
 * Test infrastructure (checker only). Drop-in replacement for the reference's
 * src/Base/ThreadPool.h (same class name and member signatures, ThreadPool.h:19-121) that runs
 * every pushed task inline, in push order, on the calling thread with thread id 0.
 *
 * The reference's multi-threaded raster lets blocks of different triangles race on the depth and
 * colour read-modify-write (RendererSoft.cpp:733-766, waited only at :337) and lets program clones
 * share one sampler LOD callback (ShaderProgramSoft.h:105-114). Running the tasks in order removes
 * both races and gives the deterministic single-threaded result the parity tests compare against.
 * This header is placed ahead of the reference sources on the include path by oracle/ref/Makefile;
 * the timed multi-threaded build does not use it.
 */
#pragma once

#include <cstddef>
#include <functional>

namespace SoftGL {

class ThreadPool {
 public:
  explicit ThreadPool(const size_t threadCnt = 1) { (void) threadCnt; }

  inline size_t getThreadCnt() const { return 1; }

  template<typename F>
  void pushTask(const F &task) {
    std::function<void(size_t)> fn(task);
    fn(0);
  }

  void waitTasksFinish() const {}
};

}  // namespace SoftGL
