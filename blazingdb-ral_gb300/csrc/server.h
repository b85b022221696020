// server.h — the served form of the expression path: a request loop over HBM-resident tables.
//
// Clients register tables (columns stay where the caller put them, in device memory) and
// filter + project queries over them, then submit requests (one run of one query).  A
// scheduler thread admits requests while the working set (resident tables plus the outputs
// and scratch of admitted requests) stays under a byte budget, and runs admitted requests in
// waves: one launch of the persistent dispatcher whose warps pull (request, chunk) work items.
// A wave carries about wave_rows rows.  Admitted requests not already in flight enter it in
// order of fewest rows left, less a credit that grows with the time they have waited, each
// with at most half of the wave; a large request is sliced over several waves (its
// look-back status words stay in its scratch between them).  So requests that arrive while a
// large one runs finish within a wave or two instead of waiting for it, and large requests
// keep advancing instead of starving under a stream of small ones.  Up to max_waves waves are in flight on their own
// streams; a request is in at most one in-flight wave at a time, so no launch ever waits on
// another.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "codegen.h"
#include "filter.h"
#include "jit.h"

namespace ral {

struct ServerTable {
    std::vector<gdf_column> cols;
    int64_t rows = 0;
    size_t bytes = 0;
};

struct ServerQuery {
    int table = -1;
    std::unique_ptr<FilterPlan> plan;
    GeneratedKernel item;
    int fn = -1;               // index in the dispatcher's function list
    size_t reserve = 0;        // output + scratch bytes of one request (every row kept)
    int64_t chunks = 0;        // work items of one request
    // the standalone fused filter kernel over the query's table (the kernel ral_filter_project
    // launches), for requests that run alone on a wave: every request over a table of at least
    // the solo threshold (`large`), and any request that finds nothing else waiting
    const void* solo = nullptr;
    bool large = false;
    std::string filter_text, project_text;  // the query's texts, for the standalone kernel
    int64_t scratch_words = 0; // scratch of one request: the larger of the chunked and solo needs
};

struct ServerRequest {
    int64_t id = 0;
    int query = -1;
    bool keep = false;         // keep the outputs for ral_server_result (else freed at completion)
    double t_submit = 0, t_launch = 0, t_done = 0;  // seconds on the server's clock
    int64_t rows_out = -1;
    int status = 0;
    std::vector<void*> out_data, out_valid;
    std::vector<int64_t> null_counts;
    void* scratch = nullptr;
    bool done = false;
    int64_t next_chunk = 0;    // chunks launched so far
    bool in_wave = false;      // part of an in-flight wave
    std::vector<uint64_t> slots;  // the request's parameter slots (after its first slice)
};

struct ServerStats {
    int64_t submitted = 0, completed = 0, waves = 0, max_wave_requests = 0;
    int64_t solo = 0;          // requests run alone on the standalone kernel
    double queue_s = 0;        // summed over completed requests: submission to first launch
    double run_s = 0;          // and first launch to completion
    size_t peak_reserved = 0;
    double busy_s = 0;         // wall time with at least one wave in flight
};

class Server {
public:
    // wave_rows: row budget of one wave (a request's slice is whole chunks; 0 = default 32M)
    Server(size_t budget_bytes, int max_waves, int max_wave_requests, int64_t wave_rows = 0);
    ~Server();
    int add_table(gdf_column* const* cols, int ncols, int* table_id);
    int add_query(int table_id, const char* filter_q, const char* project_q, int* query_id);
    // Output dtypes and mask presence of a query.
    int query_outputs(int query_id, std::vector<gdf_dtype>& dtypes, std::vector<bool>& valid) const;
    // Compiles every query's item function (host thread pool), links the dispatcher and starts
    // the scheduler thread.  Queries added later trigger a relink before their first wave.
    int start();
    // Compiles the item functions and links the dispatcher without loading it (no GPU needed).
    int debug_compile(std::string& log);
    int submit(int query_id, bool keep, int64_t* request_id);
    // Waits (up to timeout_s) for a request; fills rows out and latency (submit to completion).
    int wait(int64_t request_id, double timeout_s, int64_t* rows_out, double* latency_s);
    // A kept request's outputs (device pointers owned by the server until release).
    int result(int64_t request_id, gdf_column* out_cols, int n_out);
    int release(int64_t request_id);
    // Runs a trace: request k of query q[k] submitted at start + arrival_s[k]; blocks until all
    // are done and fills each latency and kept row count.
    int run_trace(int n, const int32_t* queries, const double* arrival_s, double* latency_s, int64_t* rows_out,
                  double* makespan_s);
    int stop();
    ServerStats stats() const;
    double now() const;

private:
    struct Wave {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        void* d_desc = nullptr;        // descs | prefix | fn | counter, one allocation
        void* h_desc = nullptr;        // pinned staging of the same
        void* h_head = nullptr;        // pinned: scratch headers copied back
        size_t desc_bytes = 0;
        std::vector<int64_t> reqs;
        std::vector<int64_t> take;     // chunks of each request in this wave
        std::vector<char> last;        // the wave runs the request's last chunk
        bool solo = false;             // one request on the standalone kernel
        bool busy = false;
        double t_launch = 0;
    };
    int ensure_linked();
    void collect_items(std::vector<GeneratedKernel>& tus, std::vector<DispatchEntry>& entries, int& stride, int& smem);
    int launch_wave(Wave& w, const std::vector<int64_t>& reqs, const std::vector<int64_t>& take);
    int launch_solo(Wave& w, int64_t request_id);
    int start_request(ServerRequest& r, cudaStream_t st);
    int prepare_solo_kernels();
    void wave_ended(Wave& w);
    void finish_wave(Wave& w);
    void loop();

    size_t budget_;
    int max_waves_, max_wave_requests_;
    std::vector<ServerTable> tables_;
    std::vector<std::unique_ptr<ServerQuery>> queries_;
    size_t tables_bytes_ = 0;
    const CompiledKernel* kernel_ = nullptr;
    int linked_queries_ = 0;
    int stride_ = 1, smem_words_ = 0, grid_ = 0;
    int device_ = 0;

    mutable std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<int64_t> pending_;      // submitted, not admitted (FIFO)
    std::vector<int64_t> active_;      // admitted, not finished
    int64_t wave_rows_ = 0;
    int slice_div_ = 2;
    std::unordered_map<int64_t, std::unique_ptr<ServerRequest>> requests_;
    int64_t next_id_ = 1;
    size_t reserved_ = 0;
    std::vector<Wave> waves_;
    std::thread thread_;
    std::atomic<bool> stop_{false};
    bool started_ = false;
    int fatal_ = 0;
    std::string fatal_msg_;
    ServerStats stats_;
    double t0_ = 0;
    double busy_since_ = -1;
    int inflight_ = 0;
    int solo_inflight_ = 0;
    int64_t solo_rows_ = 0;            // tables of at least this many rows run their requests solo
};

}  // namespace ral
