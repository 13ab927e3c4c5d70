/*
 * sst_ser.cpp -- SER v3 frame sequences (the stacking pipeline's usual
 * input) read straight into the registration + stacking path.
 *
 * The reader follows c_ser_reader (core/io/c_ser_file.h:136-174,
 * core/io/c_ser_file.cc:272-532): the 178-byte LUCAM-RECORDER header (always
 * little-endian), the reference's reading of the LittleEndian field (0 means
 * little-endian pixel data: "well-known bug with endiannes in ser file
 * format", c_ser_file.cc:304-305), its bits-per-plane extension (-32 / -64
 * for float / double, 17..32 for int32), the accepted color ids, the optional
 * trailer of per-frame 64-bit timestamps, and seek / read positions.
 *
 * sst_stack_ser streams a frame range from the file through sst_stack_frames:
 * a reader thread fills one pinned chunk buffer from the file while the GPU
 * registers and stacks the previous one. Frames are scaled by
 * 1 / 2^bits_per_plane, the stacking pipeline's conversion of integer input
 * (read_input_frame, c_image_stacking_pipeline_base.cc:270-275: integer
 * frames are converted with 1 / 2^bpp even without dark or flat frames).
 */
#include <errno.h>
#include <fcntl.h>
#include <stdint.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/serstacker_gb300.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu

namespace {

constexpr size_t kHeaderBytes = 178;

int ser_fail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

int32_t le32(const uint8_t * p)
{
  return (int32_t) ((uint32_t) p[0] | ((uint32_t) p[1] << 8) | ((uint32_t) p[2] << 16) | ((uint32_t) p[3] << 24));
}

uint64_t le64(const uint8_t * p)
{
  uint64_t v = 0;
  for( int i = 7; i >= 0; --i ) v = (v << 8) | p[i];
  return v;
}

/* bytes of one sample for the header's PixelDepthPerPlane (the reference's
 * extension: -32 float, -64 double, 17..32 int32), 0 when unsupported */
int plane_bytes(int bits)
{
  if( bits > 0 && bits <= 8 ) return 1;
  if( bits > 8 && bits <= 16 ) return 2;
  if( bits > 16 && bits <= 32 ) return 4;
  if( bits == -32 ) return 4;
  if( bits == -64 ) return 8;
  return 0;
}

int plane_depth(int bits)
{
  if( bits > 0 && bits <= 8 ) return SST_DEPTH_U8;
  if( bits > 8 && bits <= 16 ) return SST_DEPTH_U16;
  if( bits > 16 && bits <= 32 ) return SST_DEPTH_S32;
  if( bits == -32 ) return SST_DEPTH_F32;
  if( bits == -64 ) return SST_DEPTH_F64;
  return -1;
}

bool color_id_supported(int c)
{
  switch ( c ) {
  case 0:                     // MONO
  case 8: case 9: case 10: case 11:      // BAYER RGGB GRBG GBRG BGGR
  case 16: case 17: case 18: case 19:    // BAYER CYYM YCMY YMCY MYYC
  case 100: case 101:         // RGB BGR
    return true;
  }
  return false;
}

bool host_little_endian()
{
  const uint16_t one = 1;
  uint8_t b;
  memcpy(&b, &one, 1);
  return b == 1;
}

/* byte order reversal of `count` samples of `size` bytes each */
void swap_samples(void * data, size_t count, int size)
{
  uint8_t * p = (uint8_t *) data;
  for( size_t i = 0; i < count; ++i, p += size ) std::reverse(p, p + size);
}

/* read exactly `bytes` at `offset` */
bool read_at(int fd, void * dst, size_t bytes, off_t offset)
{
  uint8_t * d = (uint8_t *) dst;
  while ( bytes > 0 ) {
    const ssize_t r = pread(fd, d, bytes, offset);
    if( r < 0 ) {
      if( errno == EINTR ) continue;
      return false;
    }
    if( r == 0 ) return false;
    d += r, bytes -= (size_t) r, offset += r;
  }
  return true;
}

/* Runs body(k) for k < n on up to `threads` host threads (contiguous blocks
 * of k per thread); false when any call returned false. */
template<class F>
bool parallel_blocks(int n, int threads, F body)
{
  threads = std::max(1, std::min(threads, n));
  if( threads == 1 ) {
    for( int k = 0; k < n; ++k )
      if( !body(k) ) return false;
    return true;
  }
  std::atomic<bool> ok(true);
  std::vector<std::thread> pool;
  for( int t = 0; t < threads; ++t ) {
    const int k0 = (int) ((int64_t) n * t / threads), k1 = (int) ((int64_t) n * (t + 1) / threads);
    pool.emplace_back([&, k0, k1] {
      for( int k = k0; k < k1 && ok.load(std::memory_order_relaxed); ++k )
        if( !body(k) ) ok = false;
    });
  }
  for( std::thread & th : pool ) th.join();
  return ok;
}

/* host threads for reads of `bytes`: page-cache copies scale with threads
 * (one thread reaches about 10 GB/s); one per 32 MB, at most 16 */
int read_threads(size_t bytes)
{
  const int hw = std::max(1, (int) std::thread::hardware_concurrency());
  return (int) std::max<size_t>(1, std::min<size_t>({ (size_t) 16, (size_t) hw, bytes >> 25 }));
}

}  // namespace

struct sst_ser_reader {
  int fd = -1;
  sst_ser_info info {};
  size_t frame_bytes = 0;
  bool swap = false;                   // pixel data in the other byte order than the host's
  std::vector<uint64_t> timestamps;
  int curpos = 0;
  ~sst_ser_reader()
  {
    if( fd >= 0 ) close(fd);
  }
};

extern "C" int sst_ser_open(sst_ser_reader ** out, const char * path)
{
  if( !out || !path ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_open: NULL argument");
  *out = nullptr;
  sst_ser_reader * r = new (std::nothrow) sst_ser_reader;
  if( !r ) return ser_fail(SST_ERR_NOMEM, "out of host memory");
  r->fd = open(path, O_RDONLY);
  if( r->fd < 0 ) {
    const std::string msg = std::string("open('") + path + "') fails: " + strerror(errno);
    delete r;
    return ser_fail(SST_ERR_IO, msg);
  }
  struct stat sb;
  if( fstat(r->fd, &sb) != 0 || (size_t) sb.st_size < kHeaderBytes ) {
    delete r;
    return ser_fail(SST_ERR_IO, std::string("too small for a SER header: ") + path);
  }
  uint8_t h[kHeaderBytes];
  if( !read_at(r->fd, h, kHeaderBytes, 0) ) {
    delete r;
    return ser_fail(SST_ERR_IO, std::string("read(SER header) fails: ") + path);
  }
  if( memcmp(h, "LUCAM-RECORDER", 14) != 0 ) {
    delete r;
    return ser_fail(SST_ERR_UNSUPPORTED, std::string("not a SER file: ") + path);
  }
  sst_ser_info & in = r->info;
  in.luid = le32(h + 14);
  in.color_id = le32(h + 18);
  in.data_little_endian = le32(h + 22) == 0 ? 1 : 0;   // the field is read inverted, as the reference does
  in.width = le32(h + 26);
  in.height = le32(h + 30);
  in.bits_per_plane = le32(h + 34);
  in.frames = le32(h + 38);
  memcpy(in.observer, h + 42, 40);
  memcpy(in.instrument, h + 82, 40);
  memcpy(in.telescope, h + 122, 40);
  in.observer[40] = in.instrument[40] = in.telescope[40] = 0;
  in.date_time = le64(h + 162);
  in.date_time_utc = le64(h + 170);
  if( in.width < 1 || in.height < 1 || plane_bytes(in.bits_per_plane) == 0 ) {
    delete r;
    return ser_fail(SST_ERR_UNSUPPORTED, std::string("unsupported image size or pixel format in ") + path);
  }
  if( !color_id_supported(in.color_id) ) {
    delete r;
    return ser_fail(SST_ERR_UNSUPPORTED, std::string("unsupported ColorId in ") + path);
  }
  if( in.frames < 0 ) in.frames = 0;
  in.channels = (in.color_id == 100 || in.color_id == 101) ? 3 : 1;
  in.bytes_per_plane = plane_bytes(in.bits_per_plane);
  in.depth = plane_depth(in.bits_per_plane);
  r->frame_bytes = (size_t) in.width * in.height * in.channels * in.bytes_per_plane;
  r->swap = (in.data_little_endian != 0) != host_little_endian() && in.bytes_per_plane > 1;
  // the timestamp trailer, when the file is long enough to hold one
  const size_t ts_off = kHeaderBytes + (size_t) in.frames * r->frame_bytes;
  if( in.frames > 0 && (size_t) sb.st_size >= ts_off + (size_t) in.frames * 8 ) {
    r->timestamps.resize(in.frames);
    if( !read_at(r->fd, r->timestamps.data(), (size_t) in.frames * 8, (off_t) ts_off) ) {
      delete r;
      return ser_fail(SST_ERR_IO, std::string("read(timestamps) fails: ") + path);
    }
    if( (in.data_little_endian != 0) != host_little_endian() ) swap_samples(r->timestamps.data(), in.frames, 8);
    in.has_timestamps = 1;
  }
  *out = r;
  return SST_OK;
}

extern "C" int sst_ser_close(sst_ser_reader * r)
{
  delete r;
  return SST_OK;
}

extern "C" int sst_ser_get_info(const sst_ser_reader * r, sst_ser_info * info)
{
  if( !r || !info ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_get_info: NULL argument");
  *info = r->info;
  return SST_OK;
}

extern "C" int sst_ser_timestamps(const sst_ser_reader * r, uint64_t * ts, int n)
{
  if( !r || (!ts && n > 0) ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_timestamps: NULL argument");
  if( !r->info.has_timestamps ) return ser_fail(SST_ERR_STATE, "the SER file has no timestamps");
  const int m = std::min(n, (int) r->timestamps.size());
  memcpy(ts, r->timestamps.data(), (size_t) m * 8);
  return m;
}

extern "C" int sst_ser_curpos(const sst_ser_reader * r)
{
  return r ? r->curpos : -1;
}

extern "C" int sst_ser_seek(sst_ser_reader * r, int frame)
{
  if( !r ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_seek: NULL argument");
  if( frame < 0 ) frame = 0;
  if( frame != r->curpos ) {
    if( frame >= r->info.frames )
      return ser_fail(SST_ERR_INVALID_ARG, "invalid seek " + std::to_string(frame) + " >= FrameCount=" +
          std::to_string(r->info.frames));
    r->curpos = frame;
  }
  return SST_OK;
}

extern "C" int sst_ser_read(sst_ser_reader * r, int n, void * dst, size_t frame_stride, int * frames_read)
{
  if( frames_read ) *frames_read = 0;
  if( !r || !dst || n < 0 ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_read: invalid argument");
  if( frame_stride == 0 ) frame_stride = r->frame_bytes;
  if( frame_stride < r->frame_bytes ) return ser_fail(SST_ERR_INVALID_ARG, "frame_stride below the frame size");
  const int m = std::max(0, std::min(n, r->info.frames - r->curpos));
  uint8_t * d = (uint8_t *) dst;
  const size_t fb = r->frame_bytes;
  const off_t base = (off_t) (kHeaderBytes + (size_t) r->curpos * fb);
  const int threads = read_threads((size_t) m * fb);
  bool ok;
  if( frame_stride == fb ) {
    // contiguous frames: the byte range split into 1 MB pieces over the threads
    const size_t total = (size_t) m * fb, piece = (size_t) 1 << 20;
    const int pieces = (int) ((total + piece - 1) / piece);
    ok = parallel_blocks(pieces, threads, [&](int k) {
      const size_t o = (size_t) k * piece;
      return read_at(r->fd, d + o, std::min(piece, total - o), base + (off_t) o);
    });
  }
  else {
    ok = parallel_blocks(m, threads, [&](int k) {
      return read_at(r->fd, d + (size_t) k * frame_stride, fb, base + (off_t) ((size_t) k * fb));
    });
  }
  if( !ok ) return ser_fail(SST_ERR_IO, "read(frames " + std::to_string(r->curpos) + "..) fails or the file is truncated");
  if( r->swap ) {
    const size_t samples = fb / r->info.bytes_per_plane;
    parallel_blocks(m, threads, [&](int k) {
      swap_samples(d + (size_t) k * frame_stride, samples, r->info.bytes_per_plane);
      return true;
    });
  }
  r->curpos += m;
  if( frames_read ) *frames_read = m;
  return SST_OK;
}

/* ------------------------------------------------ streamed stacking of a file */

namespace {

struct PinnedBuf {
  void * p = nullptr;
  ~PinnedBuf()
  {
    if( p ) cudaFreeHost(p);
  }
};

}  // namespace

extern "C" int sst_stack_ser(sst_ecch * reg, sst_weighted_average * const * acc, sst_ser_reader * ser, int first,
    int count, int chunk, int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream)
{
  if( !reg || !acc || !acc[0] || !ser ) return ser_fail(SST_ERR_INVALID_ARG, "sst_stack_ser: NULL argument");
  const sst_ser_info & in = ser->info;
  const bool bayer = in.color_id >= 8 && in.color_id <= 11;
  if( in.channels != 1 || (in.color_id != 0 && !bayer) )
    return ser_fail(SST_ERR_UNSUPPORTED, "sst_stack_ser: mono or RGGB-family Bayer SER files only");
  if( in.depth != SST_DEPTH_U8 && in.depth != SST_DEPTH_U16 && in.depth != SST_DEPTH_F32 )
    return ser_fail(SST_ERR_UNSUPPORTED, "sst_stack_ser: 8-bit, 16-bit or float SER files only");
  if( bayer && in.depth != SST_DEPTH_U16 ) return ser_fail(SST_ERR_UNSUPPORTED, "sst_stack_ser: Bayer SER files must be 16-bit");
  if( bayer )
    for( int k = 1; k < 4; ++k )
      if( !acc[k] ) return ser_fail(SST_ERR_INVALID_ARG, "sst_stack_ser: a Bayer file needs four plane accumulators");
  if( first < 0 || first > in.frames ) return ser_fail(SST_ERR_INVALID_ARG, "sst_stack_ser: first frame out of range");
  if( count < 0 ) count = in.frames - first;
  count = std::min(count, in.frames - first);
  if( count == 0 ) return SST_OK;
  if( chunk <= 0 ) chunk = 256;
  // each of the two pinned buffers holds at most 512 MB of frames
  chunk = std::min(chunk, (int) std::max<size_t>(1, ((size_t) 512 << 20) / ser->frame_bytes));
  chunk = std::min(chunk, count);
  // read_input_frame: integer frames are scaled by 1 / 2^bpp
  const double scale = in.depth == SST_DEPTH_F32 ? 1.0 : 1.0 / (double) (1u << in.bits_per_plane);
  const size_t fb = ser->frame_bytes;
  PinnedBuf buf[2];
  for( int b = 0; b < 2; ++b ) {
    const cudaError_t e = cudaHostAlloc(&buf[b].p, fb * chunk, cudaHostAllocDefault);
    if( e != cudaSuccess ) return ser_fail(SST_ERR_CUDA, std::string("cudaHostAlloc failed: ") + cudaGetErrorString(e));
  }
  int rc = sst_ser_seek(ser, first);
  if( rc != SST_OK ) return rc;
  int got = 0;
  rc = sst_ser_read(ser, chunk, buf[0].p, fb, &got);
  if( rc != SST_OK ) return rc;
  int b = 0;
  for( int f0 = 0; f0 < count; f0 += chunk, b ^= 1 ) {
    const int nc = std::min(chunk, count - f0);
    if( got != nc ) return ser_fail(SST_ERR_IO, "sst_stack_ser: short read");
    // the next chunk is read from the file while this one is registered and stacked
    int next_rc = SST_OK, next_got = 0;
    const int nn = std::min(chunk, count - f0 - nc);
    std::thread reader;
    if( nn > 0 ) reader = std::thread([&, nn, b] { next_rc = sst_ser_read(ser, nn, buf[b ^ 1].p, fb, &next_got); });
    float * po = params_out ? params_out + (size_t) f0 * 12 : nullptr;
    int32_t * so = status_out ? status_out + f0 : nullptr;
    float * ro = rho_out ? rho_out + f0 : nullptr;
    float * wo = weight_out ? weight_out + f0 : nullptr;
    const int w = in.width, h = in.height;
    if( bayer )
      rc = sst_stack_bayer_frames(reg, acc, buf[b].p, nc, w, h, (size_t) w * 2, fb, scale, 0, num_passes, passes, border,
          weighting, po, so, ro, wo, stream);
    else
      rc = sst_stack_frames(reg, acc[0], buf[b].p, in.depth, nc, w, h, (size_t) w * in.bytes_per_plane, fb, scale, 0,
          num_passes, passes, border, weighting, po, so, ro, wo, stream);
    if( reader.joinable() ) reader.join();
    if( rc != SST_OK ) return rc;
    if( next_rc != SST_OK ) return next_rc;
    got = next_got;
  }
  return SST_OK;
}

/* ------------------------------------------------------------- SER output */

struct sst_ser_writer {
  int fd = -1;
  uint8_t header[kHeaderBytes] = {};
  int32_t frames = 0;
  uint64_t date_time = 0;
  size_t frame_bytes = 0;
  std::vector<uint64_t> timestamps;
};

namespace {

void put32(uint8_t * p, int32_t v)
{
  for( int i = 0; i < 4; ++i ) p[i] = (uint8_t) ((uint32_t) v >> (8 * i));
}

void put64(uint8_t * p, uint64_t v)
{
  for( int i = 0; i < 8; ++i ) p[i] = (uint8_t) (v >> (8 * i));
}

bool write_at(int fd, const void * src, size_t bytes, off_t offset)
{
  const uint8_t * s = (const uint8_t *) src;
  while ( bytes > 0 ) {
    const ssize_t r = pwrite(fd, s, bytes, offset);
    if( r < 0 ) {
      if( errno == EINTR ) continue;
      return false;
    }
    s += r, bytes -= (size_t) r, offset += r;
  }
  return true;
}

}  // namespace

extern "C" int sst_ser_writer_create(sst_ser_writer ** out, const char * path, int width, int height, int color_id,
    int bits_per_plane)
{
  if( !out || !path ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_writer_create: NULL argument");
  *out = nullptr;
  if( width < 1 || height < 1 || plane_bytes(bits_per_plane) == 0 )
    return ser_fail(SST_ERR_INVALID_ARG, "unsupported image size or PixelDepthPerPlane");
  if( !color_id_supported(color_id) ) return ser_fail(SST_ERR_INVALID_ARG, "invalid ColorId " + std::to_string(color_id));
  sst_ser_writer * w = new (std::nothrow) sst_ser_writer;
  if( !w ) return ser_fail(SST_ERR_NOMEM, "out of host memory");
  memcpy(w->header, "LUCAM-RECORDER", 14);
  put32(w->header + 18, color_id);
  // LittleEndian written as the reference's writer does: 0 on a little-endian
  // host, which its reader (and this one) takes as little-endian data
  put32(w->header + 22, host_little_endian() ? 0 : 1);
  put32(w->header + 26, width);
  put32(w->header + 30, height);
  put32(w->header + 34, bits_per_plane);
  const int channels = (color_id == 100 || color_id == 101) ? 3 : 1;
  w->frame_bytes = (size_t) width * height * channels * plane_bytes(bits_per_plane);
  w->fd = open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if( w->fd < 0 || !write_at(w->fd, w->header, kHeaderBytes, 0) ) {
    const std::string msg = std::string("create('") + path + "') fails: " + strerror(errno);
    if( w->fd >= 0 ) close(w->fd);
    delete w;
    return ser_fail(SST_ERR_IO, msg);
  }
  *out = w;
  return SST_OK;
}

extern "C" int sst_ser_write(sst_ser_writer * w, const void * frames, int n, size_t frame_stride,
    const uint64_t * timestamps)
{
  if( !w || (!frames && n > 0) || n < 0 ) return ser_fail(SST_ERR_INVALID_ARG, "sst_ser_write: invalid argument");
  if( frame_stride == 0 ) frame_stride = w->frame_bytes;
  if( frame_stride < w->frame_bytes ) return ser_fail(SST_ERR_INVALID_ARG, "frame_stride below the frame size");
  const uint8_t * s = (const uint8_t *) frames;
  for( int k = 0; k < n; ++k ) {
    const off_t at = (off_t) (kHeaderBytes + (size_t) w->frames * w->frame_bytes);
    if( !write_at(w->fd, s + (size_t) k * frame_stride, w->frame_bytes, at) )
      return ser_fail(SST_ERR_IO, std::string("write(frame) fails: ") + strerror(errno));
    const uint64_t ts = timestamps ? timestamps[k] : UINT64_MAX;
    if( w->frames == 0 ) w->date_time = ts;   // DateTime and DateTime_UTC of the first frame
    w->timestamps.push_back(ts);
    ++w->frames;
  }
  return SST_OK;
}

extern "C" int sst_ser_writer_close(sst_ser_writer * w)
{
  if( !w ) return SST_OK;
  int rc = SST_OK;
  put32(w->header + 38, w->frames);
  put64(w->header + 162, w->date_time);
  put64(w->header + 170, w->date_time);
  std::vector<uint8_t> ts(w->timestamps.size() * 8);
  for( size_t i = 0; i < w->timestamps.size(); ++i ) put64(ts.data() + 8 * i, w->timestamps[i]);
  if( !write_at(w->fd, w->header, kHeaderBytes, 0) ||
      !write_at(w->fd, ts.data(), ts.size(), (off_t) (kHeaderBytes + (size_t) w->frames * w->frame_bytes)) )
    rc = ser_fail(SST_ERR_IO, std::string("write(SER header / timestamps) fails: ") + strerror(errno));
  if( close(w->fd) != 0 && rc == SST_OK ) rc = ser_fail(SST_ERR_IO, std::string("close fails: ") + strerror(errno));
  delete w;
  return rc;
}
