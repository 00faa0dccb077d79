// Restart files of SAVE_FLOW, BACKUP_FLOW and READ_FLOW
// (src/diablo.F90:753-1072), written from and read into the resident state.
//
// The reference opens them FORM="UNFORMATTED" with sequential access, so each
// WRITE statement is one record framed by 4-byte length markers in the host's
// byte order (ifort's and gfortran's default; both build hosts here are
// little-endian).  A record longer than 2^31 - 9 bytes is split into
// subrecords: the leading marker of a subrecord is negative when another
// subrecord follows, the trailing marker negative when one precedes it.
//
//   flow file    [NX NY NZ (int32) TIME (real*8) TIME_STEP (int32)]      24 bytes
//                [CU1X CU2X CU3X CPX, each (0:NX/2, 0:NZ+1, 0:NY+1) complex*16]
//   scalar file  [NX NY NZ TIME TIME_STEP] [CTHX(:,:,:,N)]
//
// The spectral fields are stored in HBM in the same order (i fastest, then
// k, then j), so each record is the concatenation of whole device arrays and
// moves in large chunks through two pinned staging buffers: the copy of one
// chunk overlaps the file write (or read) of the other.
//
// Reading checks every record's framing and length before any device memory
// is written, so a bad file leaves the state as it was.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ek_internal.h"

namespace ek {
namespace {

constexpr int64_t kSubrecordMax = 2147483639;  // 2^31 - 9: largest subrecord payload
constexpr size_t kChunk = size_t(32) << 20;    // staging chunk
constexpr int64_t kHeaderBytes = 24;

// The subrecord limit; EKGPU_FORTRAN_SUBRECORD lowers it so that small files
// exercise the split (tests), never above the runtime's own limit.
int64_t subrecord_max() {
  const char *s = std::getenv("EKGPU_FORTRAN_SUBRECORD");
  if (!s || !*s) return kSubrecordMax;
  const long long v = std::atoll(s);
  return (v >= 1 && v < kSubrecordMax) ? (int64_t)v : kSubrecordMax;
}

struct IoError {
  std::string msg;
};

[[noreturn]] void io_fail(const std::string &path, const std::string &what) { throw IoError{path + ": " + what}; }

struct File {
  FILE *f = nullptr;
  std::string path;
  File(const char *p, const char *mode) : path(p) {
    f = std::fopen(p, mode);
    if (!f) io_fail(path, std::string("cannot open: ") + std::strerror(errno));
    std::setvbuf(f, nullptr, _IONBF, 0);  // chunks are large; no second copy through stdio
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void put(const void *b, size_t n) {
    if (n && std::fwrite(b, 1, n, f) != n) io_fail(path, std::string("write failed: ") + std::strerror(errno));
  }
  void get(void *b, size_t n) {
    if (n && std::fread(b, 1, n, f) != n) io_fail(path, "unexpected end of file");
  }
  void seek(int64_t off) {
    if (fseeko(f, (off_t)off, SEEK_SET) != 0) io_fail(path, "seek failed");
  }
  int64_t tell() { return (int64_t)ftello(f); }
  void close() {
    FILE *g = f;
    f = nullptr;
    if (std::fclose(g) != 0) io_fail(path, std::string("close failed: ") + std::strerror(errno));
  }
};

int32_t get_i32(File &f) {
  int32_t v;
  f.get(&v, 4);
  return v;
}
void put_i32(File &f, int32_t v) { f.put(&v, 4); }

// One record of `total` payload bytes, written in pieces.
class RecordWriter {
 public:
  RecordWriter(File &f, int64_t total) : f_(f), left_(total), smax_(subrecord_max()) { open_sub(); }
  void put(const void *p, size_t n) {
    const char *b = static_cast<const char *>(p);
    while (n) {
      if (sub_left_ == 0) {
        close_sub();
        open_sub();
      }
      const size_t k = (size_t)std::min<int64_t>((int64_t)n, sub_left_);
      f_.put(b, k);
      b += k;
      n -= k;
      sub_left_ -= (int64_t)k;
    }
  }
  void finish() {
    if (sub_left_ != 0 || left_ != 0) io_fail(f_.path, "record written short");
    close_sub();
  }

 private:
  void open_sub() {
    sub_len_ = std::min(left_, smax_);
    left_ -= sub_len_;
    put_i32(f_, (int32_t)(left_ > 0 ? -sub_len_ : sub_len_));
    sub_left_ = sub_len_;
  }
  void close_sub() {
    put_i32(f_, (int32_t)(first_ ? sub_len_ : -sub_len_));
    first_ = false;
  }
  File &f_;
  int64_t left_, smax_, sub_len_ = 0, sub_left_ = 0;
  bool first_ = true;
};

// Framing of one record as found in the file: the file offset and length of
// each subrecord's payload.
struct Record {
  std::vector<std::pair<int64_t, int64_t>> subs;
  int64_t bytes = 0;
};

// Walk one record from the current position, checking that the markers pair
// up and the continuation signs agree; leaves the file after the record.
Record scan_record(File &f) {
  Record r;
  for (bool first = true;; first = false) {
    const int32_t lead = get_i32(f);
    const int64_t len = lead < 0 ? -(int64_t)lead : lead;
    const int64_t off = f.tell();
    r.subs.push_back({off, len});
    r.bytes += len;
    f.seek(off + len);
    const int32_t tail = get_i32(f);
    const int64_t tlen = tail < 0 ? -(int64_t)tail : tail;
    if (tlen != len || (tail < 0) == first) io_fail(f.path, "corrupt record markers");
    if (lead >= 0) break;
  }
  return r;
}

// Reads the first bytes of a scanned record in pieces.
class RecordReader {
 public:
  RecordReader(File &f, const Record &r) : f_(f), r_(r) {}
  void get(void *p, size_t n) {
    char *b = static_cast<char *>(p);
    while (n) {
      while (in_sub_ == r_.subs[sub_].second) {
        ++sub_;
        in_sub_ = 0;
        if (sub_ >= r_.subs.size()) io_fail(f_.path, "record too short");
      }
      if (in_sub_ == 0 || !positioned_) {
        f_.seek(r_.subs[sub_].first + in_sub_);
        positioned_ = true;
      }
      const size_t k = (size_t)std::min<int64_t>((int64_t)n, r_.subs[sub_].second - in_sub_);
      f_.get(b, k);
      b += k;
      n -= k;
      in_sub_ += (int64_t)k;
    }
  }

 private:
  File &f_;
  const Record &r_;
  size_t sub_ = 0;
  int64_t in_sub_ = 0;
  bool positioned_ = false;
};

struct Header {
  int32_t nx, ny, nz, time_step;
  double time;
};

void write_header(File &f, const Dims &d, double time, int time_step) {
  unsigned char b[kHeaderBytes];
  const int32_t n[3] = {d.NX, d.NY, d.NZ};
  std::memcpy(b, n, 12);
  std::memcpy(b + 12, &time, 8);
  const int32_t ts = time_step;
  std::memcpy(b + 20, &ts, 4);
  RecordWriter w(f, kHeaderBytes);
  w.put(b, kHeaderBytes);
  w.finish();
}

Header read_header(File &f, const Record &r) {
  unsigned char b[kHeaderBytes];
  RecordReader rd(f, r);
  rd.get(b, kHeaderBytes);
  Header h;
  int32_t n[3];
  std::memcpy(n, b, 12);
  std::memcpy(&h.time, b + 12, 8);
  std::memcpy(&h.time_step, b + 20, 4);
  h.nx = n[0];
  h.ny = n[1];
  h.nz = n[2];
  return h;
}

// Two pinned staging buffers with their copy-done events.
struct Staging {
  void *buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  size_t cap;
  explicit Staging(size_t need) : cap(std::min(need, kChunk)) {
    for (int i = 0; i < 2; ++i) {
      EK_CUDA(cudaHostAlloc(&buf[i], cap, cudaHostAllocDefault));
      EK_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    }
  }
  ~Staging() {
    for (int i = 0; i < 2; ++i) {
      if (ev[i]) cudaEventSynchronize(ev[i]), cudaEventDestroy(ev[i]);
      if (buf[i]) cudaFreeHost(buf[i]);
    }
  }
};

struct Chunk {
  char *dev;
  size_t n;
};

std::vector<Chunk> chunks_of(const std::vector<cplx_t *> &fields, size_t bytes, size_t cap) {
  std::vector<Chunk> out;
  for (cplx_t *f : fields)
    for (size_t o = 0; o < bytes; o += cap) out.push_back({reinterpret_cast<char *>(f) + o, std::min(cap, bytes - o)});
  return out;
}

// Device arrays -> one record, the next chunk's copy overlapping this chunk's write.
void record_from_device(Ctx &c, File &f, const std::vector<cplx_t *> &fields) {
  const size_t bytes = c.d.nspec() * sizeof(cplx_t);
  RecordWriter w(f, (int64_t)(bytes * fields.size()));
  Staging s(bytes);
  const std::vector<Chunk> ch = chunks_of(fields, bytes, s.cap);
  auto issue = [&](size_t i) {
    EK_CUDA(cudaMemcpyAsync(s.buf[i & 1], ch[i].dev, ch[i].n, cudaMemcpyDeviceToHost, c.stream));
    EK_CUDA(cudaEventRecord(s.ev[i & 1], c.stream));
  };
  for (size_t i = 0; i < ch.size() && i < 2; ++i) issue(i);
  for (size_t i = 0; i < ch.size(); ++i) {
    EK_CUDA(cudaEventSynchronize(s.ev[i & 1]));
    w.put(s.buf[i & 1], ch[i].n);
    if (i + 2 < ch.size()) issue(i + 2);
  }
  w.finish();
}

// The first bytes of a scanned record -> device arrays.
void record_to_device(Ctx &c, File &f, const Record &r, const std::vector<cplx_t *> &fields) {
  const size_t bytes = c.d.nspec() * sizeof(cplx_t);
  RecordReader rd(f, r);
  Staging s(bytes);
  const std::vector<Chunk> ch = chunks_of(fields, bytes, s.cap);
  for (size_t i = 0; i < ch.size(); ++i) {
    if (i >= 2) EK_CUDA(cudaEventSynchronize(s.ev[i & 1]));  // the buffer's previous copy is done
    rd.get(s.buf[i & 1], ch[i].n);
    EK_CUDA(cudaMemcpyAsync(ch[i].dev, s.buf[i & 1], ch[i].n, cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaEventRecord(s.ev[i & 1], c.stream));
  }
  EK_CUDA(cudaStreamSynchronize(c.stream));
}

// A restart file opened and checked: header, dimensions, data record length.
struct Checked {
  File f;
  Header h;
  Record data;
  Checked(const char *path, const Dims &d, int64_t need, bool check_dims) : f(path, "rb") {
    const Record hr = scan_record(f);
    if (hr.bytes < kHeaderBytes) io_fail(f.path, "header record too short");
    h = read_header(f, hr);
    if (check_dims && (h.nx != d.NX || h.ny != d.NY || h.nz != d.NZ))
      io_fail(f.path, "Error: old flowfield wrong dimensions. (file " + std::to_string(h.nx) + "x" +
                          std::to_string(h.ny) + "x" + std::to_string(h.nz) + ")");
    f.seek(hr.subs.back().first + hr.subs.back().second + 4);
    data = scan_record(f);
    if (data.bytes < need) io_fail(f.path, "data record too short");
  }
};

}  // namespace

int save_flow(Ctx &c, const char *flow_path, const char *th_path) {
  try {
    File f(flow_path, "wb");
    write_header(f, c.d, c.p.time, c.p.time_step);
    record_from_device(c, f, {c.CU1, c.CU2, c.CU3, c.CP});
    f.close();
    if (th_path) {
      File g(th_path, "wb");
      write_header(g, c.d, c.p.time, c.p.time_step);
      record_from_device(c, g, {c.CTH});
      g.close();
    }
  } catch (const IoError &e) {
    c.err = e.msg;
    return EK_ERR_IO;
  }
  return EK_OK;
}

int read_flow(Ctx &c, const char *flow_path, const char *th_path) {
  try {
    const int64_t field = (int64_t)(c.d.nspec() * sizeof(cplx_t));
    // The reference checks the flow file's dimensions only; the scalar file's
    // are checked here too, since reading a record of another grid would fill
    // CTHX with a wrong layout.
    Checked fl(flow_path, c.d, 4 * field, true);
    std::vector<Checked *> all{&fl};
    std::unique_ptr<Checked> th;
    if (th_path) {
      th.reset(new Checked(th_path, c.d, field, true));
      all.push_back(th.get());
    }
    record_to_device(c, fl.f, fl.data, {c.CU1, c.CU2, c.CU3, c.CP});
    if (th) record_to_device(c, th->f, th->data, {c.CTH});
    const size_t bytes = c.d.nspec() * sizeof(cplx_t);
    for (cplx_t *f : {c.CF1, c.CF2, c.CF3, c.CFTH}) EK_CUDA(cudaMemsetAsync(f, 0, bytes, c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    // TIME and TIME_STEP: the last header read wins, as in READ_FLOW
    c.p.time = all.back()->h.time;
    c.p.time_step = all.back()->h.time_step;
    // a run started from a restart file begins with FIRST_TIME (diablo.F90:88):
    // with LES, C_DYN is recomputed in each substep of its first step
    c.les.first_time = true;
  } catch (const IoError &e) {
    c.err = e.msg;
    return EK_ERR_IO;
  }
  return EK_OK;
}

}  // namespace ek
