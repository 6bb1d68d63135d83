// handle.h -- what an h2h_graph handle holds, and the status-code wrapper
// every extern "C" entry point runs its body in.
#pragma once

#include <mutex>
#include <string>

#include "graph.h"

namespace gh {

void set_last_error(const std::string &msg);
const std::string &last_error();

// Host-buffer query staging owned by a handle.
struct HostQueryStage {
  std::mutex mu;
  int *dx = nullptr, *dy = nullptr, *dout = nullptr;
  int64_t cap = 0;
  cudaStream_t stream = nullptr, stream2 = nullptr;  // large batches alternate chunks between them
  cudaEvent_t joined = nullptr;
  int *dbad = nullptr;  // this path's own out-of-range flag (device batches on the graph never touch it)
  ~HostQueryStage() {
    cudaFree(dx); cudaFree(dy); cudaFree(dout); cudaFree(dbad);
    if (stream) cudaStreamDestroy(stream);
    if (stream2) cudaStreamDestroy(stream2);
    if (joined) cudaEventDestroy(joined);
  }
};

// Runs f, turning internal exceptions into a status code and a per-thread
// message; nothing exits the process.
template <typename F>
int guarded(F &&f) {
  try {
    f();
    return H2H_OK;
  } catch (const Error &e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    set_last_error("host allocation failed");
    return H2H_ERR_NOMEM;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return H2H_ERR_STATE;
  }
}

}  // namespace gh

struct h2h_graph {
  gh::Graph g;
  gh::HostQueryStage stage;
};
