// f3d_serve.cpp -- the serving loop: concurrent streams of planes of any
// size, bit depth and parameters on one GPU.
//
// The reference serves one clip per filter instance and lets VapourSynth call
// getFrame from many threads, serialised per instance by a mutex
// (src/fft3dcl.cpp:289, :365-368). Here one server owns the GPU work of many
// streams:
//  - admission: a stream is opened only while the device memory of all open
//    streams (engine tables and buffers, its window's spectra cache, its
//    staging planes) fits the server's HBM budget and a slot is free;
//    otherwise f3d_server_open answers F3D_E_BUSY and the caller retries once
//    another stream has closed;
//  - residency: each stream has its own engine, so its temporal-window
//    spectra (and Kalman state) stay in HBM between frames;
//  - continuous batching: one scheduler thread launches, on every pass, the
//    next output of every stream whose window frames have arrived. Streams
//    that run the fused tensor-core form are grouped by the parameters their
//    kernels take (block size, overlap, window, temporal mode, sample
//    format) into lanes of up to three streams (consecutive opens: the
//    planes of a YUV stream); each lane has one CUDA stream, and the ready
//    outputs of a lane go into one step: one launch per kernel for its
//    planes of any sizes. Lanes run concurrently with each other, as do the
//    other streams (fast or exact form, Kalman) on their own CUDA streams.
//    Streams opened while others run join the next pass;
//  - latency: an output's latency runs from the arrival of the last input
//    frame its window needs to the completion of its readback to host memory.
#include "f3d_engine_internal.hpp"
#include "fft3d_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace f3d {
void set_last_error(const char* msg);
}

namespace {

using Clock = std::chrono::steady_clock;

double now_ms() {
  return std::chrono::duration<double, std::milli>(Clock::now().time_since_epoch()).count();
}

int fail(int code, const std::string& msg) {
  static thread_local std::string m;
  m = msg;
  f3d::set_last_error(m.c_str());
  return code;
}

constexpr int kInSlots = 6;   // submitted frames a stream may hold before they are uploaded
constexpr int kOutSlots = 3;  // outputs a stream may hold before they are polled
// Shared steps of one group queued on the GPU at once. While one runs, the
// group's outputs that become ready collect for its next step (two in flight
// measured 1-2% lower capacity and a higher server-side p99 on the bench's
// serving mix).
constexpr int kMaxInflight = 1;
// Streams per lane: the three planes of a YUV stream share steps; streams of
// different lanes run concurrently.
constexpr int kLaneStreams = 3;

struct InSlot {
  uint8_t* host = nullptr;  // pinned
  int frame = -1;
  enum { FREE, RESERVED, FULL, UPLOADED } state = FREE;  // RESERVED: a submit is copying into it
  long long seq = 0;        // output launch count when the upload was queued
  double t_arrive = 0.0;
};

struct OutSlot {
  uint8_t* host = nullptr;  // pinned
  cudaEvent_t ev = nullptr;
  int frame = -1;
  long long seq = 0;
  double t_ready = 0.0, t_done = 0.0;
  bool busy = false, done = false;
};

struct Stream {
  int id = -1;
  f3d_engine* eng = nullptr;
  cudaStream_t cs = nullptr;  // the stream's own CUDA stream, or its group's (batched)
  bool own_cs = true;
  bool batched = false;       // launched in shared steps with other streams
  uint64_t gkey = 0;          // lane of a batched stream: launch key | lane index << 56
  // A batched stream copies on its own two CUDA streams, so that its copies
  // overlap its group's steps: the upload waits for the step that last read
  // the staging plane (ev_read), the step waits for the upload (ev_up) and
  // for the read-back of the previous output (last_d2h), and the read-back
  // waits for the step (ev_out).
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t ev_up = nullptr, ev_read = nullptr, ev_out = nullptr, last_d2h = nullptr;
  bool read_pending = false;
  int W = 0, H = 0, bps = 1, nframes = 0, need = 1, cur = 0, bt = 1;
  size_t row_bytes = 0, plane_bytes = 0, est_bytes = 0;
  uint8_t* d_src = nullptr;
  uint8_t* d_dst = nullptr;
  InSlot in[kInSlots];
  std::deque<OutSlot*> outs;  // launched, in frame order
  OutSlot out_pool[kOutSlots];
  int next_out = 0;           // next output frame to launch
  long long seq = 0;
  std::vector<double> arrive; // arrival time of each input frame
  std::string err;
};

void free_stream(Stream* s) {
  if (s->up) cudaStreamSynchronize(s->up);
  if (s->cs) cudaStreamSynchronize(s->cs);
  if (s->down) cudaStreamSynchronize(s->down);
  if (s->eng) f3d_engine_destroy(s->eng);
  for (auto& i : s->in)
    if (i.host) cudaFreeHost(i.host);
  for (auto& o : s->out_pool) {
    if (o.host) cudaFreeHost(o.host);
    if (o.ev) cudaEventDestroy(o.ev);
  }
  if (s->d_src) cudaFree(s->d_src);
  if (s->d_dst) cudaFree(s->d_dst);
  if (s->cs && s->own_cs) cudaStreamDestroy(s->cs);
  for (cudaStream_t c : {s->up, s->down})
    if (c) cudaStreamDestroy(c);
  for (cudaEvent_t ev : {s->ev_up, s->ev_read, s->ev_out})
    if (ev) cudaEventDestroy(ev);
  delete s;
}

// Whether a stream's engine will run the fused tensor-core form (the
// conditions of its forward and sweep: mode 1, 16x16 or 32x32 blocks, half
// overlap, not Kalman), so that it is created on its group's CUDA stream.
bool predict_batchable(int form, const f3d_internal_params& ip) {
  return form == F3D_FORM_TC && ip.bm != 0 && ip.mode == 1 && ip.bw == ip.bh && (ip.bw == 16 || ip.bw == 32) &&
         ip.ow * 2 == ip.bw &&
         ip.oh * 2 == ip.bh;
}

// Host copies of large planes (a submitted frame into its pinned slot, a
// finished output out of its slot) split by rows over a few helper threads
// and the calling thread, so that a 4K frame's copy is not one core's
// memory bandwidth.
class CopyPool {
 public:
  explicit CopyPool(int helpers) {
    for (int i = 0; i < helpers; i++) th_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> lk(mtx_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  // Rows [0, h) of `row` bytes from src (pitch sp) to dst (pitch dp).
  void copy_rows(uint8_t* dst, long long dp, const uint8_t* src, long long sp, int h, size_t row) {
    const int parts = row * h < kSplitBytes ? 1 : std::min((int)th_.size() + 1, h);
    if (parts <= 1) {
      rows(dst, dp, src, sp, 0, h, row);
      return;
    }
    std::mutex m;
    std::condition_variable done;
    int left = parts - 1;
    {
      std::lock_guard<std::mutex> lk(mtx_);
      for (int p = 1; p < parts; p++)
        jobs_.push_back(Job{dst, dp, src, sp, (int)((long long)h * p / parts), (int)((long long)h * (p + 1) / parts),
                            row, &left, &m, &done});
    }
    cv_.notify_all();
    rows(dst, dp, src, sp, 0, h / parts, row);
    std::unique_lock<std::mutex> lk(m);
    done.wait(lk, [&] { return left == 0; });
  }

 private:
  static constexpr size_t kSplitBytes = 1 << 20;
  struct Job {
    uint8_t* dst;
    long long dp;
    const uint8_t* src;
    long long sp;
    int y0, y1;
    size_t row;
    int* left;
    std::mutex* m;
    std::condition_variable* done;
  };
  static void rows(uint8_t* dst, long long dp, const uint8_t* src, long long sp, int y0, int y1, size_t row) {
    if (dp == (long long)row && sp == (long long)row) {
      std::memcpy(dst + (size_t)y0 * row, src + (size_t)y0 * row, (size_t)(y1 - y0) * row);
      return;
    }
    for (int y = y0; y < y1; y++) std::memcpy(dst + y * dp, src + y * sp, row);
  }
  void loop() {
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> lk(mtx_);
        cv_.wait(lk, [&] { return stop_ || !jobs_.empty(); });
        if (jobs_.empty()) return;  // stop_
        j = jobs_.front();
        jobs_.pop_front();
      }
      rows(j.dst, j.dp, j.src, j.sp, j.y0, j.y1, j.row);
      // The caller's mutex is held while its counter drops and it is woken,
      // so the caller cannot return (and free both) before this is done.
      std::lock_guard<std::mutex> g(*j.m);
      if (--*j.left == 0) j.done->notify_all();
    }
  }
  std::vector<std::thread> th_;
  std::mutex mtx_;
  std::condition_variable cv_;
  std::deque<Job> jobs_;
  bool stop_ = false;
};

}  // namespace

struct f3d_server {
  f3d_server_config cfg{};
  // Lanes of batched streams, by launch key and lane index: one CUDA
  // stream each, the end events of the shared steps queued on it, and the
  // open streams it holds.
  struct Group {
    cudaStream_t cs = nullptr;
    std::deque<cudaEvent_t> inflight;
    int members = 0;
  };
  std::map<uint64_t, Group> groups;
  std::deque<cudaEvent_t> spare;  // unused step events
  long long steps = 0, step_outputs = 0;
  double busy_ms = 0.0;  // scheduler passes that launched work
  int max_step = 0;
  std::mutex mtx;
  std::condition_variable work_cv, done_cv;
  std::map<int, Stream*> streams;
  int next_id = 0;
  size_t used_bytes = 0;
  std::vector<double> lat;  // per-output latency, ms
  double t_first = -1.0, t_last = 0.0;
  std::atomic<bool> stop{false};
  std::thread worker;
  CopyPool copies{3};

  void run();
  bool ready(Stream* s, int n, std::vector<int>& win);
  void launch(Stream* s, int n, const std::vector<int>& win);
  bool launch_shared();
  void step_group(std::vector<Stream*>& grp, cudaStream_t cs);
  void reap(Stream* s);
};

// Window of output n (src/fft3dcl.cpp:396-430): frames clamp(n - cur + i).
bool f3d_server::ready(Stream* s, int n, std::vector<int>& win) {
  win.clear();
  for (int i = 0; i < s->need; i++) win.push_back(std::min(std::max(n - s->cur + i, 0), s->nframes - 1));
  for (int fn : win) {
    if (f3d_has(s->eng, fn)) continue;
    bool found = false;
    for (auto& slot : s->in)
      if (slot.state == InSlot::FULL && slot.frame == fn) found = true;
    if (!found) return false;
  }
  return true;
}

void f3d_server::launch(Stream* s, int n, const std::vector<int>& win) {
  OutSlot* o = nullptr;
  for (auto& c : s->out_pool)
    if (!c.busy) {
      o = &c;
      break;
    }
  double t_ready = 0.0;
  int rc = F3D_OK;
  for (int fn : win) {
    t_ready = std::max(t_ready, s->arrive[fn]);
    if (f3d_has(s->eng, fn)) continue;
    for (auto& slot : s->in) {
      if (slot.state != InSlot::FULL || slot.frame != fn) continue;
      cudaMemcpyAsync(s->d_src, slot.host, s->plane_bytes, cudaMemcpyHostToDevice, s->cs);
      if (rc == F3D_OK) rc = f3d_forward_device(s->eng, fn, s->d_src, s->row_bytes);
      slot.state = InSlot::UPLOADED;
      slot.seq = s->seq;
      break;
    }
  }
  if (rc == F3D_OK) rc = f3d_process_device(s->eng, win.data(), (int)win.size(), s->d_dst, s->row_bytes);
  if (rc != F3D_OK && s->err.empty()) s->err = f3d_engine_error(s->eng);
  cudaMemcpyAsync(o->host, s->d_dst, s->plane_bytes, cudaMemcpyDeviceToHost, s->cs);
  cudaEventRecord(o->ev, s->cs);
  // The plugin's cache window (src/fft3dcl.cpp:457-466).
  f3d_prune(s->eng, n - s->cur - 1, n - s->cur + s->bt);
  o->busy = true;
  o->done = false;
  o->frame = n;
  o->seq = s->seq++;
  o->t_ready = t_ready;
  s->outs.push_back(o);
}

// Marks finished outputs done and frees the input slots their uploads used.
void f3d_server::reap(Stream* s) {
  for (OutSlot* o : s->outs) {
    if (o->done) continue;
    if (cudaEventQuery(o->ev) != cudaSuccess) break;  // outputs finish in order on one stream
    o->done = true;
    o->t_done = now_ms();
    lat.push_back(o->t_done - o->t_ready);
    if (t_first < 0.0) t_first = o->t_ready;
    t_last = std::max(t_last, o->t_done);
    for (auto& slot : s->in)
      if (slot.state == InSlot::UPLOADED && slot.seq <= o->seq) slot.state = InSlot::FREE;
  }
}

// One shared step per lane of batched streams whose next outputs are ready
// (their kernels take the same parameters). Returns whether anything was
// launched.
bool f3d_server::launch_shared() {
  std::map<uint64_t, std::vector<Stream*>> ready_by_group;
  std::vector<int> win;
  for (auto& kv : streams) {
    Stream* s = kv.second;
    if (!s->batched || !s->err.empty() || s->next_out >= s->nframes || (int)s->outs.size() >= kOutSlots) continue;
    if (!ready(s, s->next_out, win)) continue;
    ready_by_group[s->gkey].push_back(s);
  }
  bool any = false;
  for (auto& kv : ready_by_group) {
    Group& g = groups[kv.first];
    while (!g.inflight.empty() && cudaEventQuery(g.inflight.front()) == cudaSuccess) {
      spare.push_back(g.inflight.front());
      g.inflight.pop_front();
    }
    if ((int)g.inflight.size() >= kMaxInflight) continue;
    std::vector<Stream*>& all = kv.second;
    for (size_t i = 0; i < all.size(); i += 16) {
      std::vector<Stream*> grp(all.begin() + i, all.begin() + std::min(all.size(), i + 16));
      step_group(grp, g.cs);
    }
    any = true;
    cudaEvent_t ev = nullptr;
    if (!spare.empty()) {
      ev = spare.back();
      spare.pop_back();
    } else if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      ev = nullptr;
    }
    if (ev) {
      cudaEventRecord(ev, g.cs);
      g.inflight.push_back(ev);
    }
  }
  return any;
}

// The next output of every stream of grp in shared steps: the window frames
// not cached yet go up one per stream and step (forward only), the last
// with the outputs; then each output is copied to its host slot.
void f3d_server::step_group(std::vector<Stream*>& grp, cudaStream_t shared) {
  const int n = (int)grp.size();
  std::vector<std::vector<int>> wins(n), missing(n);
  std::vector<double> t_ready(n, 0.0);
  size_t rounds = 1;
  for (int i = 0; i < n; i++) {
    Stream* s = grp[i];
    ready(s, s->next_out, wins[i]);
    for (int fn : wins[i]) {
      t_ready[i] = std::max(t_ready[i], s->arrive[fn]);
      if (!f3d_has(s->eng, fn) && std::find(missing[i].begin(), missing[i].end(), fn) == missing[i].end())
        missing[i].push_back(fn);
    }
    rounds = std::max(rounds, missing[i].size());
  }
  f3d_engine* eng[16];
  int fns[16], nwin[16];
  const void* src[16];
  void* dst[16];
  size_t sp[16], dp[16];
  const int* wp[16];
  std::string err;
  int rc = F3D_OK;
  for (size_t r = 0; r < rounds && rc == F3D_OK; r++) {
    const bool last = r + 1 == rounds;
    for (int i = 0; i < n; i++) {
      Stream* s = grp[i];
      eng[i] = s->eng;
      fns[i] = -1;
      // The step rewrites the output plane: the previous read-back first.
      if (r == 0 && s->last_d2h) cudaStreamWaitEvent(shared, s->last_d2h, 0);
      // Entries with fewer missing frames forward theirs in the first rounds.
      if (r < missing[i].size()) {
        const int fn = missing[i][r];
        for (auto& slot : s->in) {
          if (slot.state != InSlot::FULL || slot.frame != fn) continue;
          if (s->read_pending) cudaStreamWaitEvent(s->up, s->ev_read, 0);
          cudaMemcpyAsync(s->d_src, slot.host, s->plane_bytes, cudaMemcpyHostToDevice, s->up);
          cudaEventRecord(s->ev_up, s->up);
          cudaStreamWaitEvent(shared, s->ev_up, 0);
          slot.state = InSlot::UPLOADED;
          slot.seq = s->seq;
          fns[i] = fn;
          break;
        }
      }
      src[i] = s->d_src;
      sp[i] = s->row_bytes;
      wp[i] = wins[i].data();
      nwin[i] = last ? (int)wins[i].size() : 0;
      dst[i] = s->d_dst;
      dp[i] = s->row_bytes;
    }
    rc = f3d::engines_step(eng, n, fns, src, sp, wp, nwin, dst, dp, shared, &err);
    for (int i = 0; i < n; i++)
      if (fns[i] >= 0) {
        cudaEventRecord(grp[i]->ev_read, shared);
        grp[i]->read_pending = true;
      }
  }
  if (rc == F3D_OK) {
    steps++;
    step_outputs += n;
    max_step = std::max(max_step, n);
  }
  for (int i = 0; i < n; i++) {
    Stream* s = grp[i];
    const int out_n = s->next_out++;
    OutSlot* o = nullptr;
    for (auto& c : s->out_pool)
      if (!c.busy) {
        o = &c;
        break;
      }
    if (rc != F3D_OK && s->err.empty()) s->err = err;
    cudaEventRecord(s->ev_out, shared);
    cudaStreamWaitEvent(s->down, s->ev_out, 0);
    cudaMemcpyAsync(o->host, s->d_dst, s->plane_bytes, cudaMemcpyDeviceToHost, s->down);
    cudaEventRecord(o->ev, s->down);
    s->last_d2h = o->ev;
    f3d_prune(s->eng, out_n - s->cur - 1, out_n - s->cur + s->bt);
    o->busy = true;
    o->done = false;
    o->frame = out_n;
    o->seq = s->seq++;
    o->t_ready = t_ready[i];
    s->outs.push_back(o);
  }
}

void f3d_server::run() {
  cudaSetDevice(cfg.device);
  std::vector<int> win;
  std::unique_lock<std::mutex> lk(mtx);
  while (!stop) {
    bool any = false, pending = false;
    const double t_pass = now_ms();
    for (auto& kv : streams) {
      Stream* s = kv.second;
      reap(s);
      if (s->batched) continue;
      // Continuous batching: every stream whose next window is complete
      // gets its output launched in this pass.
      while (s->next_out < s->nframes && (int)s->outs.size() < kOutSlots && ready(s, s->next_out, win)) {
        launch(s, s->next_out, win);
        s->next_out++;
        any = true;
      }
    }
    // Shared steps of the batched streams, as long as outputs are ready.
    for (int k = 0; k < kOutSlots && launch_shared(); k++) any = true;
    for (auto& kv : streams)
      for (OutSlot* o : kv.second->outs) pending |= !o->done;
    if (any) busy_ms += now_ms() - t_pass;
    done_cv.notify_all();
    if (!any) {
      // In-flight outputs are polled every 50 us; otherwise sleep until a
      // frame or a stream arrives.
      if (pending) work_cv.wait_for(lk, std::chrono::microseconds(50));
      else work_cv.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

extern "C" {

int f3d_server_create(const f3d_server_config* cfg, f3d_server** out) {
  if (!cfg || !out) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  *out = nullptr;
  if (cfg->max_streams <= 0 || cfg->hbm_budget == 0) return fail(F3D_E_PARAM, "FFT3DCL: empty server budget");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return fail(F3D_E_CUDA, "FFT3DCL: no CUDA device available");
  }
  if (cfg->device < 0 || cfg->device >= ndev) return fail(F3D_E_PARAM, "FFT3DCL: device ordinal out of range");
  auto* sv = new f3d_server();
  sv->cfg = *cfg;
  cudaSetDevice(cfg->device);
  sv->worker = std::thread([sv] { sv->run(); });
  *out = sv;
  return F3D_OK;
}

void f3d_server_destroy(f3d_server* sv) {
  if (!sv) return;
  sv->stop = true;
  sv->work_cv.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  cudaSetDevice(sv->cfg.device);
  for (auto& kv : sv->streams) free_stream(kv.second);
  for (auto& kv : sv->groups) {
    for (cudaEvent_t ev : kv.second.inflight) cudaEventDestroy(ev);
    if (kv.second.cs) cudaStreamDestroy(kv.second.cs);
  }
  for (cudaEvent_t ev : sv->spare) cudaEventDestroy(ev);
  delete sv;
}

int f3d_server_open(f3d_server* sv, const f3d_script_params* sp, const f3d_plane_geom* geom, int nframes,
                    int* sid) {
  if (!sv || !sp || !geom || !sid || nframes <= 0) return fail(F3D_E_PARAM, "FFT3DCL: bad stream arguments");
  cudaSetDevice(sv->cfg.device);
  {
    std::lock_guard<std::mutex> lk(sv->mtx);
    if ((int)sv->streams.size() >= sv->cfg.max_streams) return fail(F3D_E_BUSY, "FFT3DCL: no free stream slot");
  }
  f3d_internal_params ip{};
  int rc = f3d_validate_params(sp, geom->width, geom->height, geom->bits, &ip);
  if (rc != F3D_OK) return rc;
  auto s = std::unique_ptr<Stream, void (*)(Stream*)>(new Stream(), free_stream);
  if (predict_batchable(sv->cfg.form, ip)) {
    const uint64_t key = f3d::plane_batch_key(ip, *geom);
    std::lock_guard<std::mutex> lk(sv->mtx);
    // The first lane of this key with room (lanes are counted when a stream
    // is registered below).
    uint64_t lane = 0;
    while (lane < 255) {
      auto it = sv->groups.find(key | (lane << 56));
      if (it == sv->groups.end() || it->second.members < kLaneStreams) break;
      lane++;
    }
    s->gkey = key | (lane << 56);
    f3d_server::Group& g = sv->groups[s->gkey];
    if (!g.cs && cudaStreamCreateWithFlags(&g.cs, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      g.cs = nullptr;
      return fail(F3D_E_CUDA, "FFT3DCL: stream creation failed");
    }
    s->cs = g.cs;
    s->own_cs = false;
  } else if (cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking) != cudaSuccess) {
    return fail(F3D_E_CUDA, "FFT3DCL: stream creation failed");
  }
  f3d_options o{sv->cfg.device, sv->cfg.form, s->cs, 0};
  rc = f3d_engine_create(sp, geom, &o, &s->eng);
  if (rc != F3D_OK) return rc;
  s->batched = !s->own_cs && f3d::engine_batchable(s->eng);
  if (s->batched) {
    bool ok = cudaStreamCreateWithFlags(&s->up, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->down, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t* ev : {&s->ev_up, &s->ev_read, &s->ev_out})
      ok = ok && cudaEventCreateWithFlags(ev, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return fail(F3D_E_CUDA, "FFT3DCL: stream creation failed");
    }
  }
  f3d_engine_info info{};
  f3d_engine_get_info(s->eng, &info);
  s->W = geom->width;
  s->H = geom->height;
  s->bps = info.bytes_per_sample;
  s->row_bytes = (size_t)s->W * s->bps;
  s->plane_bytes = s->row_bytes * s->H;
  s->nframes = nframes;
  s->arrive.assign(nframes, 0.0);
  s->bt = ip.bt;
  s->need = ip.bm >= 2 ? ip.bt : 1;
  s->cur = ip.bm >= 2 ? ip.current : 0;
  // Steady state: the engine's own buffers, a cache of bt + 2 window spectra
  // plus one retired spectrum awaiting reuse, and the two staging planes.
  s->est_bytes = info.device_bytes + (size_t)(s->bt + 3) * info.spectrum_bytes + 2 * s->plane_bytes;
  {
    std::lock_guard<std::mutex> lk(sv->mtx);
    if (sv->used_bytes + s->est_bytes > sv->cfg.hbm_budget)
      return fail(F3D_E_BUSY, "FFT3DCL: the stream does not fit the server's HBM budget now");
    sv->used_bytes += s->est_bytes;
  }
  bool ok = cudaMalloc(&s->d_src, s->plane_bytes) == cudaSuccess && cudaMalloc(&s->d_dst, s->plane_bytes) == cudaSuccess;
  for (auto& i : s->in) ok = ok && cudaMallocHost(&i.host, s->plane_bytes) == cudaSuccess;
  for (auto& c : s->out_pool)
    ok = ok && cudaMallocHost(&c.host, s->plane_bytes) == cudaSuccess &&
         cudaEventCreateWithFlags(&c.ev, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(sv->mtx);
    sv->used_bytes -= s->est_bytes;
    return fail(F3D_E_NOMEM, "FFT3DCL: stream buffers could not be allocated");
  }
  std::lock_guard<std::mutex> lk(sv->mtx);
  Stream* st = s.release();
  if (st->batched || !st->own_cs) sv->groups[st->gkey].members++;
  st->id = sv->next_id++;
  *sid = st->id;
  sv->streams[st->id] = st;
  sv->work_cv.notify_all();
  return F3D_OK;
}

int f3d_server_submit(f3d_server* sv, int sid, int n, const void* src, long long pitch) {
  if (!sv || !src) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  Stream* s;
  InSlot* slot = nullptr;
  {
    std::lock_guard<std::mutex> lk(sv->mtx);
    auto it = sv->streams.find(sid);
    if (it == sv->streams.end()) return fail(F3D_E_PARAM, "FFT3DCL: unknown stream");
    s = it->second;
    if (n < 0 || n >= s->nframes) return fail(F3D_E_PARAM, "FFT3DCL: frame number out of range");
    if (pitch < (long long)s->row_bytes) return fail(F3D_E_PARAM, "FFT3DCL: pitch too small");
    for (auto& i : s->in)
      if (i.state == InSlot::FREE) {
        slot = &i;
        break;
      }
    if (!slot) return fail(F3D_E_BUSY, "FFT3DCL: the stream's input slots are full");
    slot->state = InSlot::RESERVED;  // held while the copy below runs
    slot->frame = -1;
  }
  sv->copies.copy_rows(slot->host, (long long)s->row_bytes, static_cast<const uint8_t*>(src), pitch, s->H,
                       s->row_bytes);
  {
    std::lock_guard<std::mutex> lk(sv->mtx);
    slot->frame = n;
    slot->t_arrive = now_ms();
    s->arrive[n] = slot->t_arrive;
    slot->state = InSlot::FULL;
  }
  sv->work_cv.notify_all();
  return F3D_OK;
}

int f3d_server_poll(f3d_server* sv, int sid, int* n, void* dst, long long pitch, int timeout_ms) {
  return f3d_server_poll_timed(sv, sid, n, dst, pitch, timeout_ms, nullptr, nullptr);
}

int f3d_server_poll_timed(f3d_server* sv, int sid, int* n, void* dst, long long pitch, int timeout_ms,
                          double* ready_ms, double* done_ms) {
  if (!sv || !n) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  std::unique_lock<std::mutex> lk(sv->mtx);
  auto it = sv->streams.find(sid);
  if (it == sv->streams.end()) return fail(F3D_E_PARAM, "FFT3DCL: unknown stream");
  Stream* s = it->second;
  auto front_done = [&] { return !s->outs.empty() && s->outs.front()->done; };
  if (!sv->done_cv.wait_for(lk, std::chrono::milliseconds(std::max(timeout_ms, 0)), front_done))
    return fail(F3D_E_BUSY, "FFT3DCL: no finished output yet");
  OutSlot* o = s->outs.front();
  if (!s->err.empty()) return fail(F3D_E_CUDA, s->err);
  if (dst && pitch < (long long)s->row_bytes) return fail(F3D_E_PARAM, "FFT3DCL: pitch too small");
  *n = o->frame;
  if (ready_ms) *ready_ms = o->t_ready;
  if (done_ms) *done_ms = o->t_done;
  // The copy runs without the server lock, so that the scheduler keeps
  // launching meanwhile; the slot stays busy (not reused) until it is done.
  // One thread polls a stream.
  lk.unlock();
  if (dst)
    sv->copies.copy_rows(static_cast<uint8_t*>(dst), pitch, o->host, (long long)s->row_bytes, s->H, s->row_bytes);
  lk.lock();
  s->outs.pop_front();
  o->busy = false;
  sv->work_cv.notify_all();
  return F3D_OK;
}

int f3d_server_close(f3d_server* sv, int sid) {
  if (!sv) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  Stream* s;
  {
    std::lock_guard<std::mutex> lk(sv->mtx);
    auto it = sv->streams.find(sid);
    if (it == sv->streams.end()) return fail(F3D_E_PARAM, "FFT3DCL: unknown stream");
    s = it->second;
    sv->streams.erase(it);
    sv->used_bytes -= s->est_bytes;
    if (!s->own_cs) sv->groups[s->gkey].members--;
  }
  free_stream(s);
  sv->work_cv.notify_all();
  return F3D_OK;
}

int f3d_server_get_stats(f3d_server* sv, f3d_server_stats* st) {
  if (!sv || !st) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  std::lock_guard<std::mutex> lk(sv->mtx);
  std::vector<double> v = sv->lat;
  std::memset(st, 0, sizeof *st);
  st->frames = (long long)v.size();
  st->open_streams = (int)sv->streams.size();
  st->used_bytes = sv->used_bytes;
  st->shared_steps = sv->steps;
  st->shared_outputs = sv->step_outputs;
  st->max_shared = sv->max_step;
  st->busy_ms = sv->busy_ms;
  if (v.empty()) return F3D_OK;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
  st->p50_ms = pct(0.50);
  st->p99_ms = pct(0.99);
  st->max_ms = v.back();
  double sum = 0.0;
  for (double x : v) sum += x;
  st->mean_ms = sum / v.size();
  st->seconds = (sv->t_last - sv->t_first) / 1000.0;
  return F3D_OK;
}

}  // extern "C"
