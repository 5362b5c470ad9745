// ctgpu_io.cpp -- CTSim's .pj and .if files straight to and from device
// memory, and the image utilities behind pj2if and if2 (C ABI, declared in
// include/ctgpu.h).
//
// Formats: .pj header and view records (libctsim/projections.cpp:485-546,
// :811-889), .if header, data columns and labels (libctsim/array2dfile.cpp:
// 399-640), all little-endian.
//
// A file streams through two page-locked host buffers of up to kChunk bytes
// each, on the caller's stream: while the host reads chunk k + 1 from the file
// (or writes chunk k - 1 to it), the copy engine and the unpack (pack) kernel
// work on chunk k.  Device staging for the view records is allocated
// stream-ordered and released before the call returns; the call returns
// once the data is in place.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <strings.h>
#include <vector>

#include "../../include/ctgpu.h"
#include "ctgpu_internal.h"

using namespace ctgpu;

namespace {

constexpr size_t kChunk = 8u << 20;
constexpr int kPjFixedHeader = 2 + 2 + 4 * 3 + 8 * 9 + 2 * 6 + 2;   // before the remark
constexpr int kIfHeader = 2 * 5 + 4 * 2 + 2 * 2 + 8 * 2 + 2 + 8 * 6;
constexpr uint16_t kPjSignature = 'P' * 256 + 'J';
constexpr uint16_t kIfSignature = 'I' * 256 + 'F';

int fail(int code, const std::string& msg) {
  set_last_error(msg.c_str());
  return code;
}
int ok() {
  set_last_error("");
  return CTGPU_OK;
}

#define CUDA_TRY(expr)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(CTGPU_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));   \
  } while (0)

template <class T>
void put(std::string& b, T v) {
  b.append(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <class T>
T get(const unsigned char* p) {
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

// two page-locked host buffers, two device buffers, two events; freed on exit
struct Stream2 {
  cudaStream_t st;
  unsigned char* host[2] = {nullptr, nullptr};
  unsigned char* dev = nullptr;   // 2 * devBytes (+ extra)
  cudaEvent_t ev[2] = {nullptr, nullptr};
  explicit Stream2(cudaStream_t s) : st(s) {}
  cudaError_t init(size_t hostBytes, size_t devBytes) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
      e = cudaHostAlloc(reinterpret_cast<void**>(&host[i]), hostBytes ? hostBytes : 1,
                        cudaHostAllocDefault);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess && devBytes)
      e = cudaMallocAsync(reinterpret_cast<void**>(&dev), devBytes, st);
    return e;
  }
  ~Stream2() {
    if (dev) cudaFreeAsync(dev, st);
    cudaStreamSynchronize(st);
    for (int i = 0; i < 2; i++) {
      if (host[i]) cudaFreeHost(host[i]);
      if (ev[i]) cudaEventDestroy(ev[i]);
    }
  }
};

int read_pj_header(FILE* f, const char* fn, ctgpu_pj_info* info, std::string* remark) {
  unsigned char h[kPjFixedHeader];
  if (std::fread(h, 1, sizeof(h), f) != sizeof(h))
    return fail(CTGPU_ERR_IO, std::string("Error reading header of ") + fn);
  const unsigned char* p = h;
  const uint16_t hsize = get<uint16_t>(p), sig = get<uint16_t>(p + 2);
  if (sig != kPjSignature)
    return fail(CTGPU_ERR_IO, std::string(fn) + ": not a projection file (signature)");
  std::memset(info, 0, sizeof(*info));
  ctgpu_geometry& g = info->geometry;
  g.n_view = (int32_t)get<uint32_t>(p + 4);
  g.n_det = (int32_t)get<uint32_t>(p + 8);
  g.geometry = (int32_t)get<uint32_t>(p + 12);
  double d[9];
  for (int i = 0; i < 9; i++) d[i] = get<double>(p + 16 + 8 * i);
  info->calc_time = d[0];
  g.rot_start = d[1];
  g.rot_inc = d[2];
  g.det_start = d[3];
  g.det_inc = d[4];
  g.view_diameter = d[5];
  g.focal_length = d[6];
  g.source_detector_length = d[7];
  g.fan_beam_angle = d[8];
  for (int i = 0; i < 6; i++) info->date[i] = get<uint16_t>(p + 88 + 2 * i);
  const uint16_t rlen = get<uint16_t>(p + 100);
  if (kPjFixedHeader + rlen != hsize)
    return fail(CTGPU_ERR_IO, std::string(fn) + ": header size does not match its fields");
  if (g.n_view < 0 || g.n_det < 0)
    return fail(CTGPU_ERR_IO, std::string(fn) + ": negative sizes in header");
  info->header_size = hsize;
  info->remark_length = rlen;
  if (remark) {
    remark->resize(rlen);
    if (rlen && std::fread(&(*remark)[0], 1, rlen, f) != rlen)
      return fail(CTGPU_ERR_IO, std::string("Error reading remark of ") + fn);
  }
  return CTGPU_OK;
}

int read_if_header(FILE* f, const char* fn, ctgpu_if_info* info) {
  unsigned char h[kIfHeader];
  if (std::fread(h, 1, sizeof(h), f) != sizeof(h))
    return fail(CTGPU_ERR_IO, std::string("Error reading header of ") + fn);
  const unsigned char* p = h;
  std::memset(info, 0, sizeof(*info));
  const uint16_t hsize = get<uint16_t>(p), sig = get<uint16_t>(p + 2);
  if (sig != kIfSignature)
    return fail(CTGPU_ERR_IO, std::string(fn) + ": not an image file (signature)");
  if (hsize != kIfHeader)   // array2dfile.cpp:428-432
    return fail(CTGPU_ERR_IO, std::string(fn) + ": header size does not match its fields");
  info->pixel_format = get<uint16_t>(p + 4);
  info->pixel_size = get<uint16_t>(p + 6);
  info->n_labels = get<uint16_t>(p + 8);
  info->nx = (int32_t)get<uint32_t>(p + 10);
  info->ny = (int32_t)get<uint32_t>(p + 14);
  info->data_type = get<uint16_t>(p + 18);
  info->increment_known = get<uint16_t>(p + 20);
  info->increment[0] = get<double>(p + 22);
  info->increment[1] = get<double>(p + 30);
  info->extent_known = get<uint16_t>(p + 38);
  for (int i = 0; i < 4; i++) info->extent[i] = get<double>(p + 40 + 8 * i);
  info->offset_pv = get<double>(p + 72);
  info->scale_pv = get<double>(p + 80);
  info->header_size = hsize;
  if (info->nx < 0 || info->ny < 0)
    return fail(CTGPU_ERR_IO, std::string(fn) + ": negative sizes in header");
  return CTGPU_OK;
}

void today(int32_t date[6]) {
  std::time_t t = std::time(nullptr);
  std::tm tmv;
  localtime_r(&t, &tmv);
  date[0] = tmv.tm_year + 1900;
  date[1] = tmv.tm_mon + 1;
  date[2] = tmv.tm_mday;
  date[3] = tmv.tm_hour;
  date[4] = tmv.tm_min;
  date[5] = tmv.tm_sec;
}

}  // namespace

extern "C" {

int ctgpu_pj_read_header(const char* filename, ctgpu_pj_info* info, char* remark,
                         int remark_capacity) {
  if (!filename || !info) return fail(CTGPU_ERR_INVALID, "null argument");
  File f;
  f.f = std::fopen(filename, "rb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Can not open projection file ") + filename);
  std::string r;
  int rc = read_pj_header(f.f, filename, info, &r);
  if (rc != CTGPU_OK) return rc;
  if (remark && remark_capacity > 0) {
    const size_t n = r.size() < (size_t)remark_capacity - 1 ? r.size() : (size_t)remark_capacity - 1;
    std::memcpy(remark, r.data(), n);
    remark[n] = 0;
  }
  return ok();
}

int ctgpu_pj_read_device(const char* filename, float* d_sino, int pitch, double* d_angles,
                         int* n_views_read, void* stream) {
  if (!filename || !d_sino || !d_angles) return fail(CTGPU_ERR_INVALID, "null argument");
  File f;
  f.f = std::fopen(filename, "rb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Can not open projection file ") + filename);
  ctgpu_pj_info info;
  int rc = read_pj_header(f.f, filename, &info, nullptr);
  if (rc != CTGPU_OK) return rc;
  const int nView = info.geometry.n_view, nDet = info.geometry.n_det;
  if (pitch < nDet) return fail(CTGPU_ERR_INVALID, "pitch < n_det");
  if (fseeko(f.f, (off_t)info.header_size, SEEK_SET) != 0)
    return fail(CTGPU_ERR_IO, std::string("Error seeking view data of ") + filename);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t rec = 12 + 4 * (size_t)nDet;
  const int vpc = (int)std::max<size_t>(1, kChunk / rec);
  // slots start on 256-byte boundaries (the record kernels move 16-byte words there)
  const size_t chunkBytes = (rec * (size_t)std::min(vpc, std::max(nView, 1)) + 255) & ~(size_t)255;
  Stream2 io(st);
  CUDA_TRY(io.init(chunkBytes, 2 * chunkBytes + 16));
  unsigned int* status = reinterpret_cast<unsigned int*>(io.dev + 2 * chunkBytes);
  const unsigned int init[2] = {0u, 0xffffffffu};
  CUDA_TRY(cudaMemcpyAsync(status, init, sizeof(init), cudaMemcpyHostToDevice, st));
  int done = 0;
  for (int k = 0, v0 = 0; v0 < nView; k++, v0 += vpc) {
    const int slot = k & 1;
    if (k >= 2) CUDA_TRY(cudaEventSynchronize(io.ev[slot]));
    const int nv = std::min(vpc, nView - v0);
    const size_t got = std::fread(io.host[slot], 1, rec * nv, f.f);
    const int whole = (int)(got / rec);   // projections.cpp:650-655 stops at a short record
    if (whole > 0) {
      unsigned char* dst = io.dev + slot * chunkBytes;
      CUDA_TRY(cudaMemcpyAsync(dst, io.host[slot], rec * whole, cudaMemcpyHostToDevice, st));
      CUDA_TRY(launch_pj_unpack(reinterpret_cast<const uint32_t*>(dst), whole, nDet,
                                d_sino + (size_t)v0 * pitch, pitch, d_angles + v0, v0, status,
                                st));
    }
    CUDA_TRY(cudaEventRecord(io.ev[slot], st));
    done += whole;
    if (whole < nv) break;
  }
  if (done < nView) {   // views the file does not hold: zero rows and angles
    CUDA_TRY(cudaMemsetAsync(d_sino + (size_t)done * pitch, 0,
                             sizeof(float) * (size_t)(nView - done) * pitch, st));
    CUDA_TRY(cudaMemsetAsync(d_angles + done, 0, sizeof(double) * (nView - done), st));
  }
  unsigned int hs[2];
  CUDA_TRY(cudaMemcpyAsync(hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (n_views_read) *n_views_read = done;
  if (hs[0])
    return fail(CTGPU_ERR_IO, std::string(filename) + ": " + std::to_string(hs[0]) +
                                  " view record(s) with a detector count other than the "
                                  "header's, first at view " + std::to_string(hs[1]));
  return ok();
}

int ctgpu_pj_write_device(const char* filename, const ctgpu_pj_info* info, const char* remark,
                          const float* d_sino, int pitch, const double* d_angles, void* stream) {
  if (!filename || !info || !d_sino || !d_angles) return fail(CTGPU_ERR_INVALID, "null argument");
  const ctgpu_geometry& g = info->geometry;
  const int nView = g.n_view, nDet = g.n_det;
  if (nView < 0 || nDet < 0 || pitch < nDet) return fail(CTGPU_ERR_INVALID, "bad sizes");
  const size_t rlen = remark ? std::strlen(remark) : 0;
  if (kPjFixedHeader + rlen > 65535)
    return fail(CTGPU_ERR_INVALID, "remark too long for the 16-bit header size");
  std::string h;   // projections.cpp:485-546
  put<uint16_t>(h, (uint16_t)(kPjFixedHeader + rlen));
  put<uint16_t>(h, kPjSignature);
  put<uint32_t>(h, (uint32_t)nView);
  put<uint32_t>(h, (uint32_t)nDet);
  put<uint32_t>(h, (uint32_t)g.geometry);
  for (double x : {info->calc_time, g.rot_start, g.rot_inc, g.det_start, g.det_inc,
                   g.view_diameter, g.focal_length, g.source_detector_length, g.fan_beam_angle})
    put<double>(h, x);
  for (int i = 0; i < 6; i++) put<uint16_t>(h, (uint16_t)info->date[i]);
  put<uint16_t>(h, (uint16_t)rlen);
  if (rlen) h.append(remark, rlen);
  File f;
  f.f = std::fopen(filename, "wb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Error opening file for output ") + filename);
  if (std::fwrite(h.data(), 1, h.size(), f.f) != h.size())
    return fail(CTGPU_ERR_IO, std::string("Error writing header of ") + filename);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t rec = 12 + 4 * (size_t)nDet;
  const int vpc = (int)std::max<size_t>(1, kChunk / rec);
  // slots start on 256-byte boundaries (the record kernels move 16-byte words there)
  const size_t chunkBytes = (rec * (size_t)std::min(vpc, std::max(nView, 1)) + 255) & ~(size_t)255;
  Stream2 io(st);
  CUDA_TRY(io.init(chunkBytes, 2 * chunkBytes));
  int pendingViews = 0;   // views of chunk k - 1 in slot (k - 1) & 1
  for (int k = 0, v0 = 0;; k++, v0 += vpc) {
    const int slot = k & 1;
    const int nv = v0 < nView ? std::min(vpc, nView - v0) : 0;
    if (nv > 0) {
      unsigned char* dst = io.dev + slot * chunkBytes;
      CUDA_TRY(launch_pj_pack(d_sino + (size_t)v0 * pitch, pitch, d_angles + v0, nv, nDet,
                              reinterpret_cast<uint32_t*>(dst), st));
      CUDA_TRY(cudaMemcpyAsync(io.host[slot], dst, rec * nv, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaEventRecord(io.ev[slot], st));
    }
    if (pendingViews > 0) {
      const int prev = slot ^ 1;
      CUDA_TRY(cudaEventSynchronize(io.ev[prev]));
      if (std::fwrite(io.host[prev], 1, rec * pendingViews, f.f) != rec * pendingViews)
        return fail(CTGPU_ERR_IO, std::string("Error writing view data of ") + filename);
    }
    pendingViews = nv;
    if (nv == 0) break;
  }
  if (std::fflush(f.f) != 0) return fail(CTGPU_ERR_IO, std::string("Error writing ") + filename);
  return ok();
}

int ctgpu_if_read_header(const char* filename, ctgpu_if_info* info) {
  if (!filename || !info) return fail(CTGPU_ERR_INVALID, "null argument");
  File f;
  f.f = std::fopen(filename, "rb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Can not open image file ") + filename);
  int rc = read_if_header(f.f, filename, info);
  return rc != CTGPU_OK ? rc : ok();
}

int ctgpu_if_read_labels(const char* filename, ctgpu_if_label* labels, int capacity, char* text,
                         size_t text_capacity, int* n_labels) {
  if (!filename) return fail(CTGPU_ERR_INVALID, "null argument");
  File f;
  f.f = std::fopen(filename, "rb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Can not open image file ") + filename);
  ctgpu_if_info info;
  int rc = read_if_header(f.f, filename, &info);
  if (rc != CTGPU_OK) return rc;
  // array2dfile.cpp:559-595: labels follow the real (and imaginary) columns
  const size_t planes = info.data_type == 2 ? 2 : 1;
  const long long off = (long long)info.header_size +
                        (long long)planes * info.nx * info.ny * info.pixel_size;
  if (fseeko(f.f, (off_t)off, SEEK_SET) != 0)
    return fail(CTGPU_ERR_IO, std::string("Error seeking labels of ") + filename);
  size_t used = 0;
  int n = 0;
  for (int i = 0; i < info.n_labels; i++) {
    unsigned char h[24];
    if (std::fread(h, 1, sizeof(h), f.f) != sizeof(h)) break;
    const uint16_t slen = get<uint16_t>(h + 22);
    std::string s(slen, '\0');
    if (slen && std::fread(&s[0], 1, slen, f.f) != slen) break;
    if (labels && i < capacity) {
      ctgpu_if_label& l = labels[i];
      std::memset(&l, 0, sizeof(l));
      l.type = get<uint16_t>(h);
      for (int j = 0; j < 6; j++) l.date[j] = get<uint16_t>(h + 2 + 2 * j);
      l.calc_time = get<double>(h + 14);
      l.text_length = slen;
      if (text && used + slen + 1 <= text_capacity) {
        std::memcpy(text + used, s.data(), slen);
        text[used + slen] = 0;
        l.text = text + used;
        used += slen + 1;
      }
    }
    n++;
  }
  if (n_labels) *n_labels = n;
  return ok();
}

int ctgpu_if_read_device(const char* filename, float* d_image, void* stream) {
  if (!filename || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  File f;
  f.f = std::fopen(filename, "rb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Can not open image file ") + filename);
  ctgpu_if_info info;
  int rc = read_if_header(f.f, filename, &info);
  if (rc != CTGPU_OK) return rc;
  const int ps = info.pixel_size;
  if (!((ps == 4 && info.pixel_format == 7) || (ps == 8 && info.pixel_format == 8)))
    return fail(CTGPU_ERR_UNSUPPORTED,
                std::string(filename) + ": only FP32 and FP64 images can be read to the device");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)info.nx * info.ny;
  const size_t chunk = kChunk / ps;   // pixels per chunk
  const size_t cb = std::min(chunk, std::max<size_t>(n, 1)) * ps;
  Stream2 io(st);
  CUDA_TRY(io.init(cb, ps == 8 ? 2 * cb : 0));
  for (size_t k = 0, p0 = 0; p0 < n; k++, p0 += chunk) {
    const int slot = (int)(k & 1);
    if (k >= 2) CUDA_TRY(cudaEventSynchronize(io.ev[slot]));
    const size_t np = std::min(chunk, n - p0);
    if (std::fread(io.host[slot], ps, np, f.f) != np)
      return fail(CTGPU_ERR_IO, std::string("Error reading image data of ") + filename);
    if (ps == 4) {
      CUDA_TRY(cudaMemcpyAsync(d_image + p0, io.host[slot], 4 * np, cudaMemcpyHostToDevice, st));
    } else {
      double* dst = reinterpret_cast<double*>(io.dev + slot * cb);
      CUDA_TRY(cudaMemcpyAsync(dst, io.host[slot], 8 * np, cudaMemcpyHostToDevice, st));
      CUDA_TRY(launch_f64_to_f32(dst, d_image + p0, np, st));
    }
    CUDA_TRY(cudaEventRecord(io.ev[slot], st));
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  return ok();
}

int ctgpu_if_write_device(const char* filename, const ctgpu_if_info* info,
                          const ctgpu_if_label* labels, int n_labels, const float* d_image,
                          void* stream) {
  if (!filename || !info || (!d_image && (size_t)info->nx * info->ny))
    return fail(CTGPU_ERR_INVALID, "null argument");
  if (info->nx < 0 || info->ny < 0 || n_labels < 0 || n_labels > 65535)
    return fail(CTGPU_ERR_INVALID, "bad sizes");
  std::string h;   // array2dfile.cpp:443-478, FP32 real pixels
  put<uint16_t>(h, (uint16_t)kIfHeader);
  put<uint16_t>(h, kIfSignature);
  put<uint16_t>(h, 7);   // PIXEL_FLOAT32
  put<uint16_t>(h, 4);
  put<uint16_t>(h, (uint16_t)n_labels);
  put<uint32_t>(h, (uint32_t)info->nx);
  put<uint32_t>(h, (uint32_t)info->ny);
  put<uint16_t>(h, 1);   // DATA_TYPE_REAL
  put<uint16_t>(h, (uint16_t)info->increment_known);
  put<double>(h, info->increment[0]);
  put<double>(h, info->increment[1]);
  put<uint16_t>(h, (uint16_t)info->extent_known);
  for (int i = 0; i < 4; i++) put<double>(h, info->extent[i]);
  put<double>(h, info->offset_pv);
  put<double>(h, info->scale_pv);
  File f;
  f.f = std::fopen(filename, "wb");
  if (!f.f) return fail(CTGPU_ERR_IO, std::string("Error opening file for output ") + filename);
  if (std::fwrite(h.data(), 1, h.size(), f.f) != h.size())
    return fail(CTGPU_ERR_IO, std::string("Error writing header of ") + filename);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)info->nx * info->ny;
  const size_t chunk = kChunk / 4;
  {
    Stream2 io(st);
    CUDA_TRY(io.init(std::min(chunk, std::max<size_t>(n, 1)) * 4, 0));
    size_t pending = 0;
    for (size_t k = 0, p0 = 0;; k++, p0 += chunk) {
      const int slot = (int)(k & 1);
      const size_t np = p0 < n ? std::min(chunk, n - p0) : 0;
      if (np) {
        CUDA_TRY(cudaMemcpyAsync(io.host[slot], d_image + p0, 4 * np, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaEventRecord(io.ev[slot], st));
      }
      if (pending) {
        CUDA_TRY(cudaEventSynchronize(io.ev[slot ^ 1]));
        if (std::fwrite(io.host[slot ^ 1], 4, pending, f.f) != pending)
          return fail(CTGPU_ERR_IO, std::string("Error writing image data of ") + filename);
      }
      pending = np;
      if (!np) break;
    }
  }
  std::string lb;   // array2dfile.cpp:598-640
  for (int i = 0; i < n_labels; i++) {
    const ctgpu_if_label& l = labels[i];
    const size_t len = l.text ? (l.text_length > 0 ? (size_t)l.text_length : std::strlen(l.text)) : 0;
    put<uint16_t>(lb, (uint16_t)l.type);
    int32_t date[6];
    std::memcpy(date, l.date, sizeof(date));
    if (!date[0] && !date[1] && !date[2]) today(date);
    for (int j = 0; j < 6; j++) put<uint16_t>(lb, (uint16_t)date[j]);
    put<double>(lb, l.calc_time);
    put<uint16_t>(lb, (uint16_t)(len > 65535 ? 65535 : len));
    if (len) lb.append(l.text, len > 65535 ? 65535 : len);
  }
  if (!lb.empty() && std::fwrite(lb.data(), 1, lb.size(), f.f) != lb.size())
    return fail(CTGPU_ERR_IO, std::string("Error writing labels of ") + filename);
  if (std::fflush(f.f) != 0) return fail(CTGPU_ERR_IO, std::string("Error writing ") + filename);
  return ok();
}

int ctgpu_pj_pack(const float* d_sino, int pitch, const double* d_angles, int n_view, int n_det,
                  void* d_records, void* stream) {
  if (!d_sino || !d_angles || !d_records) return fail(CTGPU_ERR_INVALID, "null argument");
  if (n_view < 0 || n_det < 0 || pitch < n_det) return fail(CTGPU_ERR_INVALID, "bad sizes");
  if (reinterpret_cast<uintptr_t>(d_records) & 3)
    return fail(CTGPU_ERR_INVALID, "d_records must be 4-byte aligned");
  CUDA_TRY(launch_pj_pack(d_sino, pitch, d_angles, n_view, n_det,
                          static_cast<uint32_t*>(d_records), (cudaStream_t)stream));
  return ok();
}

int ctgpu_pj_unpack(const void* d_records, int n_view, int n_det, float* d_sino, int pitch,
                    double* d_angles, unsigned int* d_status, void* stream) {
  if (!d_records || !d_sino || !d_angles || !d_status)
    return fail(CTGPU_ERR_INVALID, "null argument");
  if (n_view < 0 || n_det < 0 || pitch < n_det) return fail(CTGPU_ERR_INVALID, "bad sizes");
  if (reinterpret_cast<uintptr_t>(d_records) & 3)
    return fail(CTGPU_ERR_INVALID, "d_records must be 4-byte aligned");
  CUDA_TRY(launch_pj_unpack(static_cast<const uint32_t*>(d_records), n_view, n_det, d_sino, pitch,
                            d_angles, 0, d_status, (cudaStream_t)stream));
  return ok();
}

int ctgpu_sino_to_image(const float* d_sino, int pitch, int n_view, int n_det, float* d_image,
                        void* stream) {
  if (!d_sino || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  if (n_view < 0 || n_det < 0 || pitch < n_det) return fail(CTGPU_ERR_INVALID, "bad sizes");
  if ((n_view + 63) / 64 > 65535) return fail(CTGPU_ERR_INVALID, "too many views");
  CUDA_TRY(launch_sino_to_image(d_sino, pitch, n_view, n_det, d_image, (cudaStream_t)stream));
  return ok();
}

int ctgpu_image_compare_device(const float* d_a, const float* d_b, int n_images, int nx, int ny,
                               size_t image_stride, double* d_dre, void* stream) {
  if (!d_a || !d_b || !d_dre) return fail(CTGPU_ERR_INVALID, "null argument");
  if (n_images < 1 || n_images > 65535 || nx < 1 || ny < 1)
    return fail(CTGPU_ERR_INVALID, "bad sizes (the reference returns false for an empty image)");
  if ((size_t)nx * ny >= (1ull << 31)) return fail(CTGPU_ERR_INVALID, "image too large (nx * ny >= 2^31)");
  if (n_images > 1 && image_stride < (size_t)nx * ny)
    return fail(CTGPU_ERR_INVALID, "image_stride < nx * ny");
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = compare_blocks(nx, ny);
  float2* scratch = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&scratch),
                           sizeof(float2) * (size_t)n_images * nb * kCmpParts, st));
  CompareLaunch L{};
  L.a = d_a;
  L.b = d_b;
  L.strideA = L.strideB = image_stride;
  L.nx = nx;
  L.ny = ny;
  L.nImages = n_images;
  L.part = scratch;
  L.out = d_dre;
  const cudaError_t e = launch_image_compare(L, st);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, std::string("image compare: ") + cudaGetErrorString(e));
  return ok();
}

int ctgpu_image_compare(const float* d_a, const float* d_b, int n_images, int nx, int ny,
                        size_t image_stride, double* h_dre, void* stream) {
  if (!h_dre) return fail(CTGPU_ERR_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  double* out = nullptr;
  if (n_images >= 1 && n_images <= 65535)
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&out), sizeof(double) * 3 * n_images, st));
  int rc = ctgpu_image_compare_device(d_a, d_b, n_images, nx, ny, image_stride, out, stream);
  cudaError_t e = cudaSuccess;
  if (rc == CTGPU_OK)
    e = cudaMemcpyAsync(h_dre, out, sizeof(double) * 3 * n_images, cudaMemcpyDeviceToHost, st);
  if (out) cudaFreeAsync(out, st);
  const cudaError_t es = cudaStreamSynchronize(st);
  if (rc != CTGPU_OK) return rc;
  if (e == cudaSuccess) e = es;
  if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, std::string("image compare: ") + cudaGetErrorString(e));
  return ok();
}

int ctgpu_image_arith(const char* op, const float* d_a, const float* d_b, float* d_out, size_t n,
                      void* stream) {
  if (!op || !d_a || !d_b || !d_out) return fail(CTGPU_ERR_INVALID, "null argument");
  int code = -1;
  const char* names[4] = {"add", "subtract", "multiply", "divide"};
  for (int i = 0; i < 4; i++)
    if (!strcasecmp(op, names[i])) code = i;
  if (code < 0) return fail(CTGPU_ERR_INVALID, std::string("Invalid image operation ") + op);
  CUDA_TRY(launch_image_arith(code, d_a, d_b, d_out, n, (cudaStream_t)stream));
  return ok();
}

}  // extern "C"
