// Served preview loop: the GPU-resident replacement for the engine's preview
// worker (crates/engine/src/coordinator/{scheduler,worker}.rs, preview_cache/).
//
// Images are opened once: the server keeps a host copy of the decoded mosaic
// and, as device-resident cache layers, the mosaic itself, the
// full-resolution demosaiced source, the 2560-px Rec.2020 preview base and the
// render outputs. Requests are newest-wins per
// image, with the reference's ticket order (scheduler.rs:176-180: a later
// revision, or the same revision and a later sequence, replaces a pending
// request; an older one is dropped). Two lanes serve them:
//
//  * the render lane (its own thread and a highest-priority stream) renders
//    every image with a pending edit and a resident base in one batched launch
//    (run_color_batch) and reads the results back, so an edit never waits for
//    a develop to finish: its kernels are scheduled ahead of the develop's;
//  * the develop lane (lowest-priority stream) runs one develop at a time
//    (rd_develop_device + rd_spatial), publishes the new base, and queues a
//    render of it with the image's last colour settings; an edit for an image
//    whose base was evicted schedules a re-develop.
//
// The develop lane owns every allocation: admission, eviction and release of
// layers happen there. A base replaced while the render lane reads it is
// retired and released after that render completes.
//
// Admission follows the reference's logical reservations
// (crates/gpu/src/memory.rs:44-60): the resident layers and the develop's
// transient working set are charged against the byte budget before they are
// taken; when a develop does not fit, the least recently used images not in
// use lose their layers (render outputs, base, mosaic).
//
// Exports (full-resolution develop + output conversions into client buffers,
// the reference's GpuExportProcessor::render, crates/gpu/src/export/mod.rs:218)
// run on the develop lane, oldest first among develops and exports, with their
// transient working set charged against the same budget.
//
// The executor behind the policy is either the CUDA pipeline or, for host-only
// tests of the policy, a dry executor that models service times.
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
#include <set>
#include <thread>
#include <vector>

#include "rd_handles.cuh"

namespace rd {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Ticket {
  uint64_t revision = 0, sequence = 0;
};

// should_replace_preview (crates/engine/src/coordinator/scheduler.rs:176-180).
bool replaces(const Ticket& current, const Ticket& candidate) {
  return candidate.revision > current.revision ||
         (candidate.revision == current.revision && candidate.sequence >= current.sequence);
}

struct EditRequest {
  uint64_t id = 0;  // 0: a render the server queued itself (after a develop)
  Ticket ticket;
  rd_color_desc color;
  Clock::time_point submitted;
};

struct DevelopRequest {
  uint64_t id = 0;  // 0: a re-develop the server scheduled itself
  Ticket ticket;
  rd_detail_desc detail;
  rd_optics_desc optics;
  Clock::time_point submitted;
};

// A full-resolution export: develop from the resident mosaic with the image's
// current settings, the spatial pass at the crop size, then each output
// conversion into a host buffer the client keeps until the result is polled.
struct ExportRequest {
  uint64_t id = 0;
  Ticket ticket;
  rd_color_desc color;
  std::vector<rd_output_desc> outputs;
  std::vector<rd_export_file> files;  // one per output; RD_FILE_ROWS when no file is asked for
  std::vector<std::vector<uint8_t>> icc, exif;  // the files' metadata, copied at submission
  std::vector<void*> dst;
  std::vector<size_t> capacity;
  size_t largest_output = 0;  // bytes of the largest output with its file encoder's working set
  Clock::time_point submitted;
};

struct ServedImage {
  uint32_t id = 0;
  std::vector<uint16_t> mosaic;  // host copy, sensor_height rows of row_stride samples
  size_t row_stride = 0;
  rd_sensor_desc sensor{};
  rd_detail_desc detail{};
  rd_optics_desc optics{};
  uint32_t tw = 0, th = 0;
  float wb[3] = {1, 1, 1}, cam[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  // resident layers (allocated and released by the develop lane)
  uint16_t* d_mosaic = nullptr;
  rd_source* source = nullptr;  // full-resolution demosaiced, sharpened camera RGB
  rd_base* base = nullptr;
  std::vector<rd_base*> retired;  // replaced bases still read by a render in flight
  uint8_t* d_out = nullptr;
  unsigned long long* d_hist = nullptr;
  uint8_t* h_front = nullptr;  // latest rendered sRGB8 (pinned), read by clients
  uint8_t* h_back = nullptr;   // the render in flight writes here
  uint64_t hist_front[1024] = {}, hist_back[1024] = {};
  uint64_t out_revision = 0;
  bool has_output = false;
  rd_color_desc last_color{};  // colour settings of the latest served edit
  bool has_color = false;
  // pending requests
  bool has_edit = false, has_develop = false, has_export = false;
  EditRequest edit;
  DevelopRequest develop;
  ExportRequest exp;
  bool render_busy = false, develop_busy = false, closing = false;
  uint64_t last_used = 0;

  size_t mosaic_bytes() const { return sizeof(uint16_t) * mosaic.size(); }
  size_t source_bytes() const { return 12 * (size_t)sensor.crop_width * sensor.crop_height; }
  size_t base_bytes() const { return sizeof(float) * 3 * (size_t)tw * th; }
  size_t out_bytes() const { return 3 * (size_t)tw * th + 1024 * sizeof(unsigned long long); }
  size_t develop_bytes() const {
    // Transient working set of one develop + spatial pass besides the source
    // (a layer of its own): f32 mosaic, RL planes, vignetting plane, optics
    // output, tile slabs.
    return 32 * (size_t)sensor.crop_width * sensor.crop_height + ((size_t)64 << 20);
  }
  // An export's transient: the full-resolution spatial pass (vignetting plane,
  // optics output, base) and the device copy of its largest output.
  size_t export_bytes(size_t largest_output) const {
    return 32 * (size_t)sensor.crop_width * sensor.crop_height + largest_output + ((size_t)64 << 20);
  }
  bool busy() const { return render_busy || develop_busy; }
};

class Executor {
 public:
  virtual ~Executor() = default;
  // Develop lane.
  virtual Status upload(ServedImage& im) = 0;
  virtual void drop_mosaic(ServedImage& im) = 0;
  virtual Status develop_source(ServedImage& im, const DevelopRequest& rq, rd_source** src) = 0;
  virtual Status develop_base(ServedImage& im, const DevelopRequest& rq, rd_source* src, rd_base** base) = 0;
  virtual void drop_source(rd_source* src) = 0;
  virtual void drop_base(rd_base* base) = 0;
  virtual Status ensure_outputs(ServedImage& im) = 0;
  virtual void drop_outputs(ServedImage& im) = 0;
  virtual Status export_outputs(ServedImage& im, const ExportRequest& rq) = 0;
  // Render lane.
  // `bases[k]` is the base of ims[k] taken when the batch was formed.
  virtual Status render(const std::vector<ServedImage*>& ims, const std::vector<rd_base*>& bases,
                        const std::vector<const rd_color_desc*>& colors) = 0;
};

Status from_code(rd_status code, const char* what) {
  return code == RD_OK ? Status{} : Status{code, what};
}

class CudaExecutor : public Executor {
 public:
  rd_ctx* dev = nullptr;  // develop lane: lowest-priority stream, owns the layers
  rd_ctx* ren = nullptr;  // render lane: highest-priority stream, owns its staging
  void* d_stage = nullptr;
  void* h_stage = nullptr;
  int stage_cap = 0;

  Status init(int device) {
    RD_TRY(from_code(rd_ctx_create(device, 0, &dev), "develop context"));
    RD_TRY(from_code(rd_ctx_create(device, 0, &ren), "render context"));
    RD_TRY(set_stream_priority(dev->c, false));
    dev->c.yield_sms = true;  // renders get SMs within one demosaic work item
    return set_stream_priority(ren->c, true);
  }
  ~CudaExecutor() override {
    if (ren) {
      if (d_stage) rd_device_free(ren, d_stage);
      if (h_stage) rd_host_free(h_stage);
      rd_ctx_destroy(ren);
    }
    if (dev) rd_ctx_destroy(dev);
  }
  Status upload(ServedImage& im) override {
    void* p = nullptr;
    RD_TRY(from_code(rd_device_alloc(dev, im.mosaic_bytes(), &p), "mosaic allocation failed"));
    im.d_mosaic = static_cast<uint16_t*>(p);
    return from_code(rd_copy_to_device(dev, p, im.mosaic.data(), im.mosaic_bytes()), "mosaic upload failed");
  }
  void drop_mosaic(ServedImage& im) override {
    if (im.d_mosaic) rd_device_free(dev, im.d_mosaic);
    im.d_mosaic = nullptr;
  }
  Status develop_source(ServedImage& im, const DevelopRequest& rq, rd_source** src) override {
    return from_code(rd_develop_device(dev, im.d_mosaic, im.row_stride, &im.sensor, &rq.detail, nullptr, src, nullptr),
                     "develop failed");
  }
  Status develop_base(ServedImage& im, const DevelopRequest& rq, rd_source* src, rd_base** base) override {
    return from_code(rd_spatial(dev, src, &rq.optics, im.tw, im.th, im.wb, im.cam, base, nullptr),
                     "spatial pass failed");
  }
  void drop_source(rd_source* src) override {
    if (src) rd_source_release(src);
  }
  void drop_base(rd_base* base) override {
    if (base) rd_base_release(base);
  }
  Status ensure_outputs(ServedImage& im) override {
    if (im.d_out) return Status{};
    // All three buffers are allocated before any is published on the image,
    // so a failed allocation leaves the image without outputs and nothing leaks.
    void* p = nullptr;
    void* a = nullptr;
    void* b = nullptr;
    Status st = from_code(rd_device_alloc(dev, im.out_bytes(), &p), "output allocation failed");
    if (st.ok()) st = from_code(rd_host_alloc(3 * (size_t)im.tw * im.th, &a), "pinned allocation failed");
    if (st.ok()) st = from_code(rd_host_alloc(3 * (size_t)im.tw * im.th, &b), "pinned allocation failed");
    if (!st.ok()) {
      if (p) rd_device_free(dev, p);
      if (a) rd_host_free(a);
      if (b) rd_host_free(b);
      return st;
    }
    im.d_hist = static_cast<unsigned long long*>(p);
    im.d_out = reinterpret_cast<uint8_t*>(im.d_hist + 1024);
    im.h_front = static_cast<uint8_t*>(a);
    im.h_back = static_cast<uint8_t*>(b);
    return Status{};
  }
  void drop_outputs(ServedImage& im) override {
    if (im.d_hist) rd_device_free(dev, im.d_hist);
    if (im.h_front) rd_host_free(im.h_front);
    if (im.h_back) rd_host_free(im.h_back);
    im.d_hist = nullptr;
    im.d_out = nullptr;
    im.h_front = im.h_back = nullptr;
    im.has_output = false;
  }
  Status export_outputs(ServedImage& im, const ExportRequest& rq) override {
    rd_base* base = nullptr;
    RD_TRY(from_code(rd_spatial(dev, im.source, &im.optics, im.sensor.crop_width, im.sensor.crop_height, im.wb,
                                im.cam, &base, nullptr),
                     "export spatial pass failed"));
    rd_status st = RD_OK;
    for (size_t k = 0; k < rq.outputs.size() && st == RD_OK; ++k) {
      if (rq.files[k].format == RD_FILE_ROWS)
        st = rd_render_output(dev, base, &rq.color, &rq.outputs[k], rq.dst[k], rq.capacity[k], nullptr, nullptr,
                              nullptr);
      else
        st = export_file(base, rq, k);
    }
    rd_base_release(base);
    return from_code(st, "export output failed");
  }
  // Output k rendered into device rows, encoded on the device, and the file
  // copied into the client's buffer.
  rd_status export_file(rd_base* base, const ExportRequest& rq, size_t k) {
    const rd_output_desc& out = rq.outputs[k];
    const rd_export_file& f = rq.files[k];
    uint32_t ow = 0, oh = 0, bpp = 0;
    rd_status st = rd_output_dimensions((uint32_t)base->W, (uint32_t)base->H, &out, &ow, &oh, &bpp);
    if (st != RD_OK) return st;
    const size_t rows = (size_t)ow * oh * bpp;
    const uint64_t bound = f.format == RD_FILE_PNG ? rd_png_bound(ow, oh, out.format == RD_OUTPUT_SRGB16 ? 16 : 8,
                                                                  f.icc_len, f.exif_len)
                                                   : rd_jpeg_bound(ow, oh, f.icc_len, f.exif_len);
    void *d_rows = nullptr, *d_file = nullptr, *d_size = nullptr;
    st = rd_device_alloc(dev, rows, &d_rows);
    if (st == RD_OK) st = rd_device_alloc(dev, bound, &d_file);
    if (st == RD_OK) st = rd_device_alloc(dev, 16, &d_size);
    if (st == RD_OK) st = rd_render_output_device(dev, base, &rq.color, &out, d_rows, nullptr, nullptr, nullptr);
    if (st == RD_OK) {
      uint8_t* file = static_cast<uint8_t*>(d_file);
      uint64_t* size_at = static_cast<uint64_t*>(d_size);
      st = f.format == RD_FILE_PNG
               ? rd_encode_png_device(dev, d_rows, ow, oh, 3ull * ow, out.format == RD_OUTPUT_SRGB16 ? 16 : 8, f.icc,
                                      f.icc_len, f.exif, f.exif_len, file, bound, size_at)
               : rd_encode_jpeg_device(dev, static_cast<const uint8_t*>(d_rows), ow, oh, 3ull * ow, f.quality, f.icc,
                                       f.icc_len, f.exif, f.exif_len, file, bound, size_at);
    }
    uint64_t size = 0;
    if (st == RD_OK) st = rd_copy_to_host(dev, &size, d_size, sizeof(size));
    if (st == RD_OK) {
      if (f.file_bytes) *f.file_bytes = size;
      st = size > rq.capacity[k] ? RD_INVALID_DIMENSIONS : rd_copy_to_host(dev, rq.dst[k], d_file, size);
    }
    if (d_size) rd_device_free(dev, d_size);
    if (d_file) rd_device_free(dev, d_file);
    if (d_rows) rd_device_free(dev, d_rows);
    return st;
  }
  Status render(const std::vector<ServedImage*>& ims, const std::vector<rd_base*>& bases,
                const std::vector<const rd_color_desc*>& colors) override {
    const int n = (int)ims.size();
    if (n > stage_cap) {
      if (d_stage) rd_device_free(ren, d_stage);
      if (h_stage) rd_host_free(h_stage);
      d_stage = h_stage = nullptr;
      stage_cap = 0;
      const size_t bytes = color_batch_staging_bytes(std::max(n, 16));
      RD_TRY(from_code(rd_device_alloc(ren, bytes, &d_stage), "staging allocation failed"));
      RD_TRY(from_code(rd_host_alloc(bytes, &h_stage), "staging allocation failed"));
      stage_cap = std::max(n, 16);
    }
    std::vector<ColorBatchItem> items(n);
    for (int k = 0; k < n; ++k) {
      items[k].rgb = bases[k]->rgb;
      items[k].width = bases[k]->W;
      items[k].height = bases[k]->H;
      items[k].color = colors[k];
      items[k].srgb = ims[k]->d_out;
      items[k].hist = ims[k]->d_hist;
    }
    Context& c = ren->c;
    cudaSetDevice(c.device);
    RD_TRY(run_color_batch(c, items.data(), n, d_stage, h_stage));
    for (int k = 0; k < n; ++k) {
      RD_CUDA_TRY(cudaMemcpyAsync(ims[k]->h_back, ims[k]->d_out, 3 * (size_t)ims[k]->tw * ims[k]->th,
                                  cudaMemcpyDeviceToHost, c.stream));
      RD_CUDA_TRY(cudaMemcpyAsync(ims[k]->hist_back, ims[k]->d_hist, sizeof(ims[k]->hist_back),
                                  cudaMemcpyDeviceToHost, c.stream));
    }
    return check_kernel_error(c, "served render");
  }
};

// Models the pipeline's service times without a device, for host-only tests of
// the admission and scheduling policy. A render writes the edit's exposure
// (x10) into the output so tests can tell which request was served.
class DryExecutor : public Executor {
 public:
  std::atomic<uint32_t> develop_us{2000}, render_us{200};
  Status upload(ServedImage& im) override {
    im.d_mosaic = reinterpret_cast<uint16_t*>(im.mosaic.data());  // marks the layer resident
    return Status{};
  }
  void drop_mosaic(ServedImage& im) override { im.d_mosaic = nullptr; }
  Status develop_source(ServedImage&, const DevelopRequest&, rd_source** src) override {
    std::this_thread::sleep_for(std::chrono::microseconds(develop_us / 2));
    *src = new rd_source{};  // marks the layer resident
    return Status{};
  }
  Status develop_base(ServedImage&, const DevelopRequest&, rd_source*, rd_base** base) override {
    std::this_thread::sleep_for(std::chrono::microseconds(develop_us - develop_us / 2));
    *base = new rd_base{};
    return Status{};
  }
  void drop_source(rd_source* src) override { delete src; }
  void drop_base(rd_base* base) override { delete base; }
  Status ensure_outputs(ServedImage& im) override {
    if (im.h_front) return Status{};
    const size_t n = 3 * (size_t)im.tw * im.th;
    im.h_front = new uint8_t[n]();
    im.h_back = new uint8_t[n]();
    im.d_out = im.h_back;  // marks the layer resident
    return Status{};
  }
  void drop_outputs(ServedImage& im) override {
    delete[] im.h_front;
    delete[] im.h_back;
    im.h_front = im.h_back = im.d_out = nullptr;
    im.has_output = false;
  }
  Status export_outputs(ServedImage&, const ExportRequest& rq) override {
    std::this_thread::sleep_for(std::chrono::microseconds(develop_us));
    const uint8_t v = (uint8_t)(rq.color.exposure_ev * 10.0f);
    for (size_t k = 0; k < rq.dst.size(); ++k) {
      std::memset(rq.dst[k], v, rq.capacity[k]);
      if (rq.files[k].format != RD_FILE_ROWS && rq.files[k].file_bytes) *rq.files[k].file_bytes = rq.capacity[k];
    }
    return Status{};
  }
  Status render(const std::vector<ServedImage*>& ims, const std::vector<rd_base*>&,
                const std::vector<const rd_color_desc*>& colors) override {
    std::this_thread::sleep_for(std::chrono::microseconds(render_us));
    for (size_t k = 0; k < ims.size(); ++k) {
      const uint8_t v = (uint8_t)(colors[k]->exposure_ev * 10.0f);
      std::memset(ims[k]->h_back, v, 3 * (size_t)ims[k]->tw * ims[k]->th);
      for (int b = 0; b < 1024; ++b) ims[k]->hist_back[b] = 0;
      ims[k]->hist_back[v] = (uint64_t)ims[k]->tw * ims[k]->th;
    }
    return Status{};
  }
};

}  // namespace
}  // namespace rd

struct rd_server {
  std::mutex mu;
  std::condition_variable render_cv, develop_cv, result_cv;
  std::map<uint32_t, std::unique_ptr<rd::ServedImage>> images;
  std::deque<rd_server_result> results;
  rd_server_stats stats{};
  uint64_t budget = 0, resident = 0, sequence = 0, next_request = 1, lru_clock = 0;
  bool stop = false, rendering = false, developing = false;
  std::unique_ptr<rd::Executor> exec;
  rd::DryExecutor* dry = nullptr;
  std::thread render_thread, develop_thread;

  // -------------------------------------------------------------- accounting
  size_t layers(const rd::ServedImage& im) const {
    return (im.d_mosaic ? im.mosaic_bytes() : 0) + (im.source ? im.source_bytes() : 0) +
           (im.base ? im.base_bytes() : 0) + (im.d_out ? im.out_bytes() : 0);
  }
  void charge(int64_t delta) {
    resident = (uint64_t)((int64_t)resident + delta);
    stats.resident_bytes = resident;
    stats.peak_resident_bytes = std::max(stats.peak_resident_bytes, resident);
  }
  // Develop lane only.
  void drop_layers(rd::ServedImage& im) {
    const size_t before = layers(im);
    exec->drop_outputs(im);
    exec->drop_base(im.base);
    im.base = nullptr;
    for (rd_base* b : im.retired) exec->drop_base(b);
    im.retired.clear();
    exec->drop_source(im.source);
    im.source = nullptr;
    exec->drop_mosaic(im);
    charge(-(int64_t)before);
  }
  // Makes room for `need` more bytes by evicting the least recently used idle
  // images other than `keep`; false when even that is not enough.
  bool admit(uint64_t need, const rd::ServedImage* keep) {
    if (budget == 0) return true;
    while (resident + need > budget) {
      rd::ServedImage* victim = nullptr;
      for (auto& kv : images) {
        rd::ServedImage& im = *kv.second;
        if (&im == keep || im.busy() || layers(im) == 0) continue;
        if (!victim || im.last_used < victim->last_used) victim = &im;
      }
      if (!victim) return false;
      drop_layers(*victim);
      stats.evictions++;
    }
    return true;
  }

  // --------------------------------------------------------------- results
  void push_result(uint64_t id, uint32_t image, int kind, rd_status st, uint64_t revision,
                   rd::Clock::time_point submitted, rd::Clock::time_point started, rd::Clock::time_point done,
                   uint32_t batch) {
    if (id == 0) return;  // a request the server made itself
    rd_server_result r{};
    r.request_id = id;
    r.image_id = image;
    r.kind = kind;
    r.status = st;
    r.revision = revision;
    r.queue_ms = rd::ms_between(submitted, started);
    r.service_ms = rd::ms_between(started, done);
    r.latency_ms = rd::ms_between(submitted, done);
    r.batch_size = batch;
    results.push_back(r);
    if (st == RD_OK) stats.completed++;
    else if (st == RD_CANCELLED) stats.coalesced++;
    else stats.failed++;
    result_cv.notify_all();
  }
  void fail_edit(rd::ServedImage& im, rd_status st) {
    const auto now = rd::Clock::now();
    push_result(im.edit.id, im.id, 0, st, im.edit.ticket.revision, im.edit.submitted, now, now, 0);
    im.has_edit = false;
  }

  // ------------------------------------------------------------ render lane
  bool renderable(const rd::ServedImage& im) const {
    return im.has_edit && !im.closing && !im.render_busy && im.base && im.d_out;
  }
  bool render_work() const {
    for (auto& kv : images)
      if (renderable(*kv.second)) return true;
    return false;
  }
  void serve_edits(std::unique_lock<std::mutex>& lk) {
    std::vector<rd::ServedImage*> batch;
    std::vector<rd_base*> bases;
    std::vector<rd::EditRequest> reqs;
    for (auto& kv : images) {
      rd::ServedImage& im = *kv.second;
      if (!renderable(im)) continue;
      batch.push_back(&im);
      bases.push_back(im.base);
      reqs.push_back(im.edit);
      im.has_edit = false;
      im.render_busy = true;
      im.last_used = ++lru_clock;
    }
    if (batch.empty()) return;
    std::vector<const rd_color_desc*> colors;
    for (const rd::EditRequest& rq : reqs) colors.push_back(&rq.color);
    const auto started = rd::Clock::now();
    lk.unlock();
    const rd::Status st = exec->render(batch, bases, colors);
    lk.lock();
    const auto done = rd::Clock::now();
    stats.batches++;
    stats.batched_edits += batch.size();
    bool retire = false;
    for (size_t k = 0; k < batch.size(); ++k) {
      rd::ServedImage& im = *batch[k];
      im.render_busy = false;
      retire = retire || !im.retired.empty() || im.closing;
      if (st.ok()) {
        std::swap(im.h_front, im.h_back);
        std::memcpy(im.hist_front, im.hist_back, sizeof(im.hist_front));
        im.out_revision = reqs[k].ticket.revision;
        im.has_output = true;
        im.last_color = reqs[k].color;
        im.has_color = true;
      }
      push_result(reqs[k].id, im.id, 0, st.ok() ? RD_OK : st.code, reqs[k].ticket.revision, reqs[k].submitted,
                  started, done, (uint32_t)batch.size());
    }
    if (retire) develop_cv.notify_all();
  }
  void render_loop() {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      render_cv.wait(lk, [&] { return stop || render_work(); });
      if (stop) break;
      rendering = true;
      serve_edits(lk);
      rendering = false;
      result_cv.notify_all();
    }
  }

  // ----------------------------------------------------------- develop lane
  bool develop_work() const {
    for (auto& kv : images) {
      const rd::ServedImage& im = *kv.second;
      if (im.busy()) continue;
      if (im.closing || im.has_develop || im.has_export || !im.retired.empty()) return true;
      if (im.has_edit && (!im.base || !im.d_out)) return true;  // needs a (re-)develop first
    }
    return false;
  }
  void housekeeping() {
    for (auto it = images.begin(); it != images.end();) {
      rd::ServedImage& im = *it->second;
      if (im.busy()) {
        ++it;
        continue;
      }
      for (rd_base* b : im.retired) exec->drop_base(b);
      im.retired.clear();
      if (im.closing) {
        drop_layers(im);
        it = images.erase(it);
        continue;
      }
      if (im.has_edit && (!im.base || !im.d_out) && !im.has_develop) {
        // Evicted: develop again with the current settings, then render the edit.
        im.has_develop = true;
        im.develop.id = 0;
        im.develop.ticket = im.edit.ticket;
        im.develop.detail = im.detail;
        im.develop.optics = im.optics;
        im.develop.submitted = im.edit.submitted;
        stats.redeveloped++;
      }
      ++it;
    }
  }
  // The oldest pending develop or export.
  void serve_develop(std::unique_lock<std::mutex>& lk) {
    rd::ServedImage* target = nullptr;
    bool is_export = false;
    rd::Clock::time_point oldest{};
    for (auto& kv : images) {
      rd::ServedImage& im = *kv.second;
      if (im.closing || im.busy()) continue;
      if (im.has_develop && (!target || im.develop.submitted < oldest)) {
        target = &im;
        is_export = false;
        oldest = im.develop.submitted;
      }
      if (im.has_export && !im.has_develop && (!target || im.exp.submitted < oldest)) {
        // A pending develop of the same image goes first: the export uses its settings.
        target = &im;
        is_export = true;
        oldest = im.exp.submitted;
      }
    }
    if (!target) return;
    if (is_export) return serve_export(lk, *target);
    rd::ServedImage& im = *target;
    const rd::DevelopRequest rq = im.develop;
    im.has_develop = false;
    im.develop_busy = true;
    im.last_used = ++lru_clock;
    const auto started = rd::Clock::now();
    // The new source and base coexist with the old ones until they are published.
    uint64_t need = im.develop_bytes() + im.source_bytes() + im.base_bytes();
    if (!im.d_mosaic) need += im.mosaic_bytes();
    if (!im.d_out) need += im.out_bytes();
    rd::Status st;
    if (!admit(need, &im)) st = rd::Status{RD_OVER_BUDGET, "develop does not fit the budget"};
    if (st.ok() && !im.d_mosaic) {
      st = exec->upload(im);
      if (st.ok()) charge((int64_t)im.mosaic_bytes());
    }
    if (st.ok() && !im.d_out) {
      st = exec->ensure_outputs(im);
      if (st.ok()) charge((int64_t)im.out_bytes());
    }
    rd_base* base = nullptr;
    rd_source* src = nullptr;
    if (st.ok()) {
      lk.unlock();
      st = exec->develop_source(im, rq, &src);
      if (st.ok()) st = exec->develop_base(im, rq, src, &base);
      lk.lock();
    }
    if (!st.ok() && src) {
      exec->drop_source(src);
      src = nullptr;
    }
    if (st.ok()) {
      // The demosaiced source of the current settings stays resident.
      if (im.source) exec->drop_source(im.source);
      else charge((int64_t)im.source_bytes());
      im.source = src;
      // Publish the new base; the old one goes when no render reads it.
      if (im.base) {
        if (im.render_busy) im.retired.push_back(im.base);
        else exec->drop_base(im.base);
      } else {
        charge((int64_t)im.base_bytes());
      }
      im.base = base;
      im.detail = rq.detail;
      im.optics = rq.optics;
      if (!im.has_edit && im.has_color) {
        // Show the new develop with the latest colour settings.
        im.edit.id = 0;
        im.edit.ticket = rq.ticket;
        im.edit.color = im.last_color;
        im.edit.submitted = rd::Clock::now();
        im.has_edit = true;
      }
    }
    im.develop_busy = false;
    push_result(rq.id, im.id, 1, st.ok() ? RD_OK : st.code, rq.ticket.revision, rq.submitted, started,
                rd::Clock::now(), 1);
    if (!st.ok() && rq.id == 0 && im.has_edit) fail_edit(im, st.code);  // its edit waited on it
    render_cv.notify_all();
  }
  void serve_export(std::unique_lock<std::mutex>& lk, rd::ServedImage& im) {
    const rd::ExportRequest rq = im.exp;
    im.has_export = false;
    im.develop_busy = true;
    im.last_used = ++lru_clock;
    const auto started = rd::Clock::now();
    const uint64_t transient = im.export_bytes(rq.largest_output);
    uint64_t need = transient;
    if (!im.d_mosaic) need += im.mosaic_bytes();
    if (!im.source) need += im.develop_bytes() + im.source_bytes();
    rd::Status st;
    if (!admit(need, &im)) st = rd::Status{RD_OVER_BUDGET, "export does not fit the budget"};
    if (st.ok() && !im.d_mosaic) {
      st = exec->upload(im);
      if (st.ok()) charge((int64_t)im.mosaic_bytes());
    }
    if (st.ok() && !im.source) {
      // Evicted or never kept: develop the source with the current settings.
      rd::DevelopRequest dq;
      dq.detail = im.detail;
      dq.optics = im.optics;
      rd_source* src = nullptr;
      lk.unlock();
      st = exec->develop_source(im, dq, &src);
      lk.lock();
      if (st.ok()) {
        im.source = src;
        charge((int64_t)im.source_bytes());
      }
    }
    if (st.ok()) {
      // The transient is charged while the export runs, so concurrent
      // admissions see it.
      charge((int64_t)transient);
      lk.unlock();
      st = exec->export_outputs(im, rq);
      lk.lock();
      charge(-(int64_t)transient);
    }
    im.develop_busy = false;
    stats.exports++;
    push_result(rq.id, im.id, 2, st.ok() ? RD_OK : st.code, rq.ticket.revision, rq.submitted, started,
                rd::Clock::now(), 1);
  }
  void develop_loop() {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      develop_cv.wait(lk, [&] { return stop || develop_work(); });
      if (stop) break;
      developing = true;
      const uint64_t before = stats.completed + stats.failed + stats.coalesced + stats.evictions + stats.redeveloped;
      housekeeping();
      serve_develop(lk);
      housekeeping();
      developing = false;
      result_cv.notify_all();
      render_cv.notify_all();
      // Pending work that cannot progress yet (an image busy in the render
      // lane) must not spin with the lock held.
      if (stats.completed + stats.failed + stats.coalesced + stats.evictions + stats.redeveloped == before)
        develop_cv.wait_for(lk, std::chrono::milliseconds(1));
    }
  }
  void wake() {
    render_cv.notify_all();
    develop_cv.notify_all();
  }
  bool idle() const { return !rendering && !developing && !render_work() && !develop_work() && !pending(); }
  bool pending() const {
    for (auto& kv : images)
      if (kv.second->has_edit || kv.second->has_develop || kv.second->has_export || kv.second->busy()) return true;
    return false;
  }
};

// ------------------------------------------------------------------ C ABI
extern "C" {

rd_status rd_server_create(int device, uint64_t budget_bytes, rd_server** out) {
  if (!out) return RD_INVALID_INPUT;
  *out = nullptr;
  auto* s = new (std::nothrow) rd_server();
  if (!s) return RD_OVER_BUDGET;
  s->budget = budget_bytes;
  s->stats.budget_bytes = budget_bytes;
  if (device < 0) {
    auto dry = std::make_unique<rd::DryExecutor>();
    s->dry = dry.get();
    s->exec = std::move(dry);
  } else {
    // The server does its own admission; the contexts' budgets are left open.
    auto cu = std::make_unique<rd::CudaExecutor>();
    const rd::Status st = cu->init(device);
    if (!st.ok()) {
      delete s;
      return st.code;
    }
    s->exec = std::move(cu);
  }
  s->render_thread = std::thread([s] { s->render_loop(); });
  s->develop_thread = std::thread([s] { s->develop_loop(); });
  *out = s;
  return RD_OK;
}

rd_status rd_server_set_dry_timing(rd_server* s, uint32_t develop_us, uint32_t render_us) {
  if (!s || !s->dry) return RD_INVALID_INPUT;
  s->dry->develop_us = develop_us;
  s->dry->render_us = render_us;
  return RD_OK;
}

void rd_server_destroy(rd_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->wake();
  if (s->render_thread.joinable()) s->render_thread.join();
  if (s->develop_thread.joinable()) s->develop_thread.join();
  for (auto& kv : s->images) s->drop_layers(*kv.second);
  s->images.clear();
  s->exec.reset();
  delete s;
}

rd_status rd_server_open(rd_server* s, uint32_t image_id, const uint16_t* mosaic, size_t row_stride,
                         const rd_sensor_desc* sensor, const rd_detail_desc* detail, const rd_optics_desc* optics,
                         uint32_t target_width, uint32_t target_height, const float wb_gains[3],
                         const float camera_to_rec2020[9], uint64_t* request_id) {
  if (!s || !mosaic || !sensor || !detail || !optics || !wb_gains || !camera_to_rec2020) return RD_INVALID_INPUT;
  if (target_width == 0 || target_height == 0 || row_stride < sensor->sensor_width) return RD_INVALID_DIMENSIONS;
  auto im = std::make_unique<rd::ServedImage>();
  im->id = image_id;
  im->mosaic.assign(mosaic, mosaic + row_stride * (size_t)sensor->sensor_height);
  im->row_stride = row_stride;
  im->sensor = *sensor;
  im->detail = *detail;
  im->optics = *optics;
  im->tw = target_width;
  im->th = target_height;
  std::memcpy(im->wb, wb_gains, sizeof(im->wb));
  std::memcpy(im->cam, camera_to_rec2020, sizeof(im->cam));
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it != s->images.end() && !it->second->closing) return RD_INVALID_INPUT;  // already open
  if (it != s->images.end()) return RD_SYNCHRONIZATION;  // still closing: retry
  // The first develop, as a request of revision 0.
  im->has_develop = true;
  im->develop.id = s->next_request++;
  im->develop.ticket = {0, ++s->sequence};
  im->develop.detail = *detail;
  im->develop.optics = *optics;
  im->develop.submitted = rd::Clock::now();
  if (request_id) *request_id = im->develop.id;
  s->stats.requested++;
  s->images[image_id] = std::move(im);
  s->wake();
  return RD_OK;
}

rd_status rd_server_close_image(rd_server* s, uint32_t image_id) {
  if (!s) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it == s->images.end() || it->second->closing) return RD_INVALID_INPUT;
  rd::ServedImage& im = *it->second;
  const auto now = rd::Clock::now();
  if (im.has_edit) s->push_result(im.edit.id, im.id, 0, RD_CANCELLED, im.edit.ticket.revision, im.edit.submitted, now, now, 0);
  if (im.has_develop)
    s->push_result(im.develop.id, im.id, 1, RD_CANCELLED, im.develop.ticket.revision, im.develop.submitted, now, now, 0);
  if (im.has_export)
    s->push_result(im.exp.id, im.id, 2, RD_CANCELLED, im.exp.ticket.revision, im.exp.submitted, now, now, 0);
  im.has_edit = im.has_develop = im.has_export = false;
  im.closing = true;
  s->wake();
  return RD_OK;
}

rd_status rd_server_submit_edit(rd_server* s, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                                uint64_t* request_id) {
  if (!s || !color) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it == s->images.end() || it->second->closing) return RD_INVALID_INPUT;
  rd::ServedImage& im = *it->second;
  rd::EditRequest rq;
  rq.id = s->next_request++;
  rq.ticket = {revision, ++s->sequence};
  rq.color = *color;
  rq.submitted = rd::Clock::now();
  if (request_id) *request_id = rq.id;
  s->stats.requested++;
  if (im.has_edit) {
    if (!rd::replaces(im.edit.ticket, rq.ticket)) {
      // An older request than the one pending: dropped (scheduler.rs:62-71).
      s->push_result(rq.id, im.id, 0, RD_CANCELLED, revision, rq.submitted, rq.submitted, rq.submitted, 0);
      return RD_OK;
    }
    s->push_result(im.edit.id, im.id, 0, RD_CANCELLED, im.edit.ticket.revision, im.edit.submitted, rq.submitted,
                   rq.submitted, 0);
  }
  im.edit = rq;
  im.has_edit = true;
  s->wake();
  return RD_OK;
}

rd_status rd_server_submit_develop(rd_server* s, uint32_t image_id, uint64_t revision, const rd_detail_desc* detail,
                                   const rd_optics_desc* optics, uint64_t* request_id) {
  if (!s || !detail || !optics) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it == s->images.end() || it->second->closing) return RD_INVALID_INPUT;
  rd::ServedImage& im = *it->second;
  rd::DevelopRequest rq;
  rq.id = s->next_request++;
  rq.ticket = {revision, ++s->sequence};
  rq.detail = *detail;
  rq.optics = *optics;
  rq.submitted = rd::Clock::now();
  if (request_id) *request_id = rq.id;
  s->stats.requested++;
  if (im.has_develop) {
    if (!rd::replaces(im.develop.ticket, rq.ticket)) {
      s->push_result(rq.id, im.id, 1, RD_CANCELLED, revision, rq.submitted, rq.submitted, rq.submitted, 0);
      return RD_OK;
    }
    s->push_result(im.develop.id, im.id, 1, RD_CANCELLED, im.develop.ticket.revision, im.develop.submitted,
                   rq.submitted, rq.submitted, 0);
  }
  im.develop = rq;
  im.has_develop = true;
  s->wake();
  return RD_OK;
}

static rd_status submit_export(rd_server* s, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                               const rd_output_desc* outputs, const rd_export_file* files, int32_t n_outputs,
                               void* const* dst, const size_t* capacities, uint64_t* request_id) {
  if (!s || !color || !outputs || !dst || !capacities || n_outputs <= 0) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it == s->images.end() || it->second->closing) return RD_INVALID_INPUT;
  rd::ServedImage& im = *it->second;
  rd::ExportRequest rq;
  for (int32_t k = 0; k < n_outputs; ++k) {
    uint32_t ow = 0, oh = 0, bpp = 0;
    const rd_status st = rd_output_dimensions(im.sensor.crop_width, im.sensor.crop_height, &outputs[k], &ow, &oh, &bpp);
    if (st != RD_OK) return st;
    const size_t bytes = (size_t)ow * oh * bpp;
    rd_export_file f{};
    if (files) f = files[k];
    size_t need = bytes, working = bytes;
    if (f.format == RD_FILE_PNG || f.format == RD_FILE_JPEG) {
      const bool png = f.format == RD_FILE_PNG;
      if ((f.icc_len && !f.icc) || (f.exif_len && !f.exif)) return RD_INVALID_INPUT;
      if (png ? !rd::png_metadata_ok(f.icc_len, f.exif_len) : !rd::jpeg_metadata_ok(f.icc_len, f.exif_len))
        return RD_INVALID_INPUT;
      if (png ? (outputs[k].format != RD_OUTPUT_SRGB8 && outputs[k].format != RD_OUTPUT_SRGB16)
              : (outputs[k].format != RD_OUTPUT_SRGB8 || f.quality < 1 || f.quality > 100))
        return RD_INVALID_INPUT;
      need = png ? rd_png_bound(ow, oh, outputs[k].format == RD_OUTPUT_SRGB16 ? 16 : 8, f.icc_len, f.exif_len)
                 : rd_jpeg_bound(ow, oh, f.icc_len, f.exif_len);
      if (need == 0) return RD_INVALID_DIMENSIONS;
      // Rows, the file, and the encoder's scratch (at most three times the rows).
      working = bytes + need + 3 * bytes;
    } else if (f.format != RD_FILE_ROWS) {
      return RD_INVALID_INPUT;
    }
    if (!dst[k] || capacities[k] < need) return RD_INVALID_DIMENSIONS;
    rq.icc.emplace_back(f.icc ? f.icc : nullptr, f.icc ? f.icc + f.icc_len : nullptr);
    rq.exif.emplace_back(f.exif ? f.exif : nullptr, f.exif ? f.exif + f.exif_len : nullptr);
    rq.outputs.push_back(outputs[k]);
    rq.files.push_back(f);
    rq.dst.push_back(dst[k]);
    rq.capacity.push_back(capacities[k]);
    rq.largest_output = std::max(rq.largest_output, working);
  }
  for (size_t k = 0; k < rq.files.size(); ++k) {  // the files read the request's own copies
    rq.files[k].icc = rq.icc[k].empty() ? nullptr : rq.icc[k].data();
    rq.files[k].exif = rq.exif[k].empty() ? nullptr : rq.exif[k].data();
  }
  rq.id = s->next_request++;
  rq.ticket = {revision, ++s->sequence};
  rq.color = *color;
  rq.submitted = rd::Clock::now();
  if (request_id) *request_id = rq.id;
  s->stats.requested++;
  if (im.has_export) {
    if (!rd::replaces(im.exp.ticket, rq.ticket)) {
      s->push_result(rq.id, im.id, 2, RD_CANCELLED, revision, rq.submitted, rq.submitted, rq.submitted, 0);
      return RD_OK;
    }
    s->push_result(im.exp.id, im.id, 2, RD_CANCELLED, im.exp.ticket.revision, im.exp.submitted, rq.submitted,
                   rq.submitted, 0);
  }
  im.exp = std::move(rq);
  im.has_export = true;
  s->wake();
  return RD_OK;
}

rd_status rd_server_submit_export(rd_server* s, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                                  const rd_output_desc* outputs, int32_t n_outputs, void* const* dst,
                                  const size_t* capacities, uint64_t* request_id) {
  return submit_export(s, image_id, revision, color, outputs, nullptr, n_outputs, dst, capacities, request_id);
}

rd_status rd_server_submit_export_files(rd_server* s, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                                        const rd_output_desc* outputs, const rd_export_file* files, int32_t n_outputs,
                                        void* const* dst, const size_t* capacities, uint64_t* request_id) {
  if (!files) return RD_INVALID_INPUT;
  return submit_export(s, image_id, revision, color, outputs, files, n_outputs, dst, capacities, request_id);
}

int32_t rd_server_poll(rd_server* s, rd_server_result* out, int32_t max_results, int32_t wait_ms) {
  if (!s || !out || max_results <= 0) return 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->results.empty() && wait_ms > 0)
    s->result_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->results.empty(); });
  int32_t n = 0;
  while (n < max_results && !s->results.empty()) {
    out[n++] = s->results.front();
    s->results.pop_front();
  }
  return n;
}

rd_status rd_server_read_output(rd_server* s, uint32_t image_id, uint8_t* srgb, uint64_t* hist, uint64_t* revision) {
  if (!s) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->images.find(image_id);
  if (it == s->images.end()) return RD_INVALID_INPUT;
  const rd::ServedImage& im = *it->second;
  if (!im.has_output) return RD_READBACK;
  if (srgb) std::memcpy(srgb, im.h_front, 3 * (size_t)im.tw * im.th);
  if (hist) std::memcpy(hist, im.hist_front, sizeof(im.hist_front));
  if (revision) *revision = im.out_revision;
  return RD_OK;
}

rd_status rd_server_get_stats(rd_server* s, rd_server_stats* out) {
  if (!s || !out) return RD_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->resident_bytes = s->resident;
  out->budget_bytes = s->budget;
  return RD_OK;
}

rd_status rd_server_drain(rd_server* s, int32_t wait_ms) {
  if (!s) return RD_INVALID_INPUT;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool idle = s->result_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return s->idle(); });
  return idle ? RD_OK : RD_SYNCHRONIZATION;
}

}  // extern "C"
