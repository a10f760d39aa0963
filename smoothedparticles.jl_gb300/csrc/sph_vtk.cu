// sph_vtk.cu -- ParaView frame export without stalling the step loop:
// save_frame! / new_pvd_file / save_pvd_file of src/IO.jl:15-75.
//
// A frame is gathered on the system's stream (the same field kernel as
// sph_get_field: reference particle order, vectors as n x 3) into one of two
// device slots together with the device-resident particle count, copied on a
// separate stream into the slot's pinned host buffer, and written by a host
// thread as <dir>/frame<k>.vtp (VTK XML PolyData, raw appended binary, one
// vertex cell per particle: what WriteVTK writes for MeshCell(PolyData.Verts(),
// [i])).  The caller's stream only carries the gather; the copy and the file
// write overlap the following steps.  sph_vtk_close writes <dir>/result.pvd
// (the frame collection) once every frame is on disk.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <filesystem>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sph_launch.h"
#include "sph_system.h"
#include "sphgpu.h"

using namespace sphgpu;

namespace {

constexpr int kSlots = 2;

struct FieldInfo {
  const char* name;
  const char* vtk_type;
  int comps;
  int bytes;  // per component
};

FieldInfo field_info(int f) {
  switch (f) {
    case SPH_FIELD_X: return {"x", "Float64", 3, 8};
    case SPH_FIELD_V: return {"v", "Float64", 3, 8};
    case SPH_FIELD_A: return {"a", "Float64", 3, 8};
    case SPH_FIELD_XSPH: return {"xsph", "Float64", 3, 8};
    case SPH_FIELD_RHO: return {"rho", "Float64", 1, 8};
    case SPH_FIELD_RHO_REF: return {"rho_ref", "Float64", 1, 8};
    case SPH_FIELD_P: return {"P", "Float64", 1, 8};
    case SPH_FIELD_TYPE: return {"type", "Int32", 1, 4};
    case SPH_FIELD_OID: return {"oid", "Int64", 1, 8};
    case SPH_FIELD_KEY: return {"key", "Int64", 1, 8};
    default: return {nullptr, nullptr, 0, 0};
  }
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

struct Job {
  int slot;
  int frame;
  unsigned fields;
  int cap;              // rows the slot's arrays hold
  cudaEvent_t copied;   // the slot's host buffer is complete
};

}  // namespace

struct sph_vtk {
  sph_system* sys = nullptr;
  std::string dir;
  cudaStream_t copy = nullptr;
  void* dbuf[kSlots] = {};
  void* hbuf[kSlots] = {};
  size_t bytes = 0;     // size of each slot
  bool busy[kSlots] = {};
  cudaEvent_t gathered[kSlots] = {};
  cudaEvent_t copied[kSlots] = {};
  int next_slot = 0;
  int frames = 0;
  std::vector<std::pair<int, double>> written;  // (frame, time) on disk
  std::vector<double> times;
  std::deque<Job> jobs;
  std::mutex mu;
  std::condition_variable cv;
  std::thread writer;
  bool stop = false;
  std::string err;
};

namespace {

// Layout of a slot: [count (int, 256 B)] then each field in SPH_FIELD order.
size_t slot_bytes(unsigned fields, int cap) {
  size_t b = 256;
  for (int f = SPH_FIELD_X; f <= SPH_FIELD_KEY; ++f)
    if (f == SPH_FIELD_X || (fields & (1u << f))) {
      const FieldInfo fi = field_info(f);
      b += align256((size_t)cap * fi.comps * fi.bytes);
    }
  return b;
}

bool write_frame(const std::string& path, const char* base, unsigned fields, int cap) {
  const int n = *(const int*)base;
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return false;
  // appended blocks: Points, PointData arrays, connectivity, offsets
  struct Block {
    const void* data;
    size_t bytes;
  };
  std::vector<Block> blocks;
  std::vector<std::string> xml_fields;
  size_t off = 0, pos = 256;
  const char* xdata = nullptr;
  std::vector<int64_t> conn((size_t)n), offs((size_t)n);
  for (int i = 0; i < n; ++i) {
    conn[i] = i;
    offs[i] = i + 1;
  }
  for (int f = SPH_FIELD_X; f <= SPH_FIELD_KEY; ++f) {
    const bool want = f == SPH_FIELD_X || (fields & (1u << f));
    if (!want) continue;
    const FieldInfo fi = field_info(f);
    const char* data = base + pos;
    pos += align256((size_t)cap * fi.comps * fi.bytes);
    if (f == SPH_FIELD_X) {
      xdata = data;
      if (!(fields & (1u << SPH_FIELD_X))) continue;
    }
    char line[256];
    std::snprintf(line, sizeof line,
                  "        <DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" "
                  "format=\"appended\" offset=\"%%zu\"/>\n",
                  fi.vtk_type, fi.name, fi.comps);
    xml_fields.push_back(line);
    blocks.push_back({data, (size_t)n * fi.comps * fi.bytes});
  }
  // offsets of the blocks: Points first, then the point data, then the verts
  std::vector<size_t> boff;
  const size_t pts_bytes = (size_t)n * 3 * 8;
  boff.push_back(off);
  off += 8 + pts_bytes;
  for (const Block& b : blocks) {
    boff.push_back(off);
    off += 8 + b.bytes;
  }
  const size_t conn_off = off;
  off += 8 + (size_t)n * 8;
  const size_t offs_off = off;
  std::fprintf(fp,
               "<?xml version=\"1.0\"?>\n"
               "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" "
               "header_type=\"UInt64\">\n"
               "  <PolyData>\n"
               "    <Piece NumberOfPoints=\"%d\" NumberOfVerts=\"%d\" NumberOfLines=\"0\" "
               "NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n"
               "      <PointData>\n",
               n, n);
  for (size_t i = 0; i < blocks.size(); ++i) std::fprintf(fp, xml_fields[i].c_str(), boff[i + 1]);
  std::fprintf(fp,
               "      </PointData>\n"
               "      <Points>\n"
               "        <DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\" "
               "format=\"appended\" offset=\"%zu\"/>\n"
               "      </Points>\n"
               "      <Verts>\n"
               "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" "
               "offset=\"%zu\"/>\n"
               "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" "
               "offset=\"%zu\"/>\n"
               "      </Verts>\n"
               "    </Piece>\n"
               "  </PolyData>\n"
               "  <AppendedData encoding=\"raw\">\n   _",
               boff[0], conn_off, offs_off);
  bool ok = true;
  auto put = [&](const void* d, size_t nb) {
    const uint64_t h = nb;
    ok = ok && std::fwrite(&h, 8, 1, fp) == 1;
    if (nb) ok = ok && std::fwrite(d, 1, nb, fp) == nb;
  };
  put(xdata, pts_bytes);
  for (const Block& b : blocks) put(b.data, b.bytes);
  put(conn.data(), (size_t)n * 8);
  put(offs.data(), (size_t)n * 8);
  std::fprintf(fp, "\n  </AppendedData>\n</VTKFile>\n");
  ok = ok && std::fclose(fp) == 0;
  return ok;
}

void writer_loop(sph_vtk* v) {
  cudaSetDevice(v->sys->device);
  for (;;) {
    Job j;
    {
      std::unique_lock<std::mutex> lk(v->mu);
      v->cv.wait(lk, [&] { return v->stop || !v->jobs.empty(); });
      if (v->jobs.empty()) return;
      j = v->jobs.front();
    }
    bool ok = cudaEventSynchronize(j.copied) == cudaSuccess;
    std::string path = v->dir + "/frame" + std::to_string(j.frame) + ".vtp";
    if (ok) ok = write_frame(path, (const char*)v->hbuf[j.slot], j.fields, j.cap);
    {
      std::lock_guard<std::mutex> lk(v->mu);
      v->jobs.pop_front();
      v->busy[j.slot] = false;
      if (ok)
        v->written.push_back({j.frame, v->times[j.frame]});
      else if (v->err.empty())
        v->err = "cannot write " + path;
    }
    v->cv.notify_all();
  }
}

void free_slots(sph_vtk* v) {
  for (int i = 0; i < kSlots; ++i) {
    if (v->dbuf[i]) cudaFree(v->dbuf[i]);
    if (v->hbuf[i]) cudaFreeHost(v->hbuf[i]);
    v->dbuf[i] = v->hbuf[i] = nullptr;
  }
  v->bytes = 0;
}

}  // namespace

extern "C" {

int sph_vtk_open(sph_system* s, const char* dir, sph_vtk** out) {
  if (!s || !dir || !out) return SPH_ERR_ARG;
  *out = nullptr;
  std::error_code ec;
  std::filesystem::create_directories(dir, ec);  // new_pvd_file: mkpath
  if (ec) return system_fail(s, SPH_ERR_ARG, ("cannot create directory " + std::string(dir)).c_str());
  DeviceGuard guard(s->device);
  sph_vtk* v = new sph_vtk();
  v->sys = s;
  v->dir = dir;
  bool ok = cudaStreamCreateWithFlags(&v->copy, cudaStreamNonBlocking) == cudaSuccess;
  for (int i = 0; i < kSlots && ok; ++i)
    ok = cudaEventCreateWithFlags(&v->gathered[i], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&v->copied[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    sph_vtk_close(v);
    return system_fail(s, SPH_ERR_CUDA, "cannot create the export stream / events");
  }
  v->writer = std::thread(writer_loop, v);
  *out = v;
  return SPH_OK;
}

int sph_vtk_save_frame(sph_vtk* v, unsigned fields, double time, int32_t* frame) {
  if (!v) return SPH_ERR_ARG;
  const unsigned valid = 0x7feu;  // bits SPH_FIELD_X .. SPH_FIELD_KEY
  if (fields & ~valid) return SPH_ERR_ARG;  // nothing queued, the series stays usable
  sph_system* s = v->sys;
  DeviceGuard guard(s->device);
  const int cap = s->n_host;
  const size_t need = slot_bytes(fields, cap > 0 ? cap : 1);
  int slot;
  {
    std::unique_lock<std::mutex> lk(v->mu);
    if (!v->err.empty()) return SPH_ERR_CUDA;
    // wait for a free slot (the writer frees one when its file is on disk)
    v->cv.wait(lk, [&] { return !v->busy[v->next_slot]; });
    slot = v->next_slot;
    if (need > v->bytes) {
      // grow both slots: wait until neither is in use
      v->cv.wait(lk, [&] { return !v->busy[0] && !v->busy[1]; });
      free_slots(v);
      for (int i = 0; i < kSlots; ++i) {
        if (cudaMalloc(&v->dbuf[i], need) != cudaSuccess ||
            cudaMallocHost(&v->hbuf[i], need) != cudaSuccess) {
          cudaGetLastError();
          free_slots(v);
          v->err = "cannot allocate the frame buffers";
          return SPH_ERR_NOMEM;
        }
      }
      v->bytes = need;
    }
    v->busy[slot] = true;
    v->next_slot = (slot + 1) % kSlots;
  }
  // gather on the system's stream: count, then the fields in reference order
  char* d = (char*)v->dbuf[slot];
  cudaError_t e = cudaMemcpyAsync(d, s->b.d_n, sizeof(int), cudaMemcpyDeviceToDevice, s->stream);
  size_t pos = 256;
  for (int f = SPH_FIELD_X; f <= SPH_FIELD_KEY && e == cudaSuccess; ++f) {
    if (f != SPH_FIELD_X && !(fields & (1u << f))) continue;
    const FieldInfo fi = field_info(f);
    if (cap > 0) e = launch_field(system_ctx(s), s->cur, s->k, s->b, cap, f, 0, d + pos);
    pos += align256((size_t)cap * fi.comps * fi.bytes);
  }
  if (e == cudaSuccess) e = cudaEventRecord(v->gathered[slot], s->stream);
  // copy on the export stream, behind the gather only
  if (e == cudaSuccess) e = cudaStreamWaitEvent(v->copy, v->gathered[slot], 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(v->hbuf[slot], d, pos, cudaMemcpyDeviceToHost, v->copy);
  if (e == cudaSuccess) e = cudaEventRecord(v->copied[slot], v->copy);
  if (e != cudaSuccess) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(v->mu);
    v->busy[slot] = false;
    v->err = std::string("frame export: ") + cudaGetErrorString(e);
    return SPH_ERR_CUDA;
  }
  {
    std::lock_guard<std::mutex> lk(v->mu);
    const int k = v->frames++;
    v->times.push_back(time);
    v->jobs.push_back({slot, k, fields, cap, v->copied[slot]});
    if (frame) *frame = k;
  }
  v->cv.notify_all();
  return SPH_OK;
}

int sph_vtk_close(sph_vtk* v) {
  if (!v) return SPH_ERR_ARG;
  if (v->writer.joinable()) {
    {
      std::lock_guard<std::mutex> lk(v->mu);
      v->stop = true;
    }
    v->cv.notify_all();
    v->writer.join();  // the writer drains the queue first
  }
  int rc = v->err.empty() ? SPH_OK : SPH_ERR_CUDA;
  // save_pvd_file: the collection of the frames on disk
  const std::string pvd = v->dir + "/result.pvd";
  FILE* fp = std::fopen(pvd.c_str(), "w");
  if (fp) {
    std::fprintf(fp,
                 "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"1.0\" "
                 "byte_order=\"LittleEndian\">\n  <Collection>\n");
    for (const auto& w : v->written)
      std::fprintf(fp, "    <DataSet timestep=\"%.17g\" group=\"\" part=\"0\" file=\"frame%d.vtp\"/>\n",
                   w.second, w.first);
    std::fprintf(fp, "  </Collection>\n</VTKFile>\n");
    if (std::fclose(fp) != 0) rc = SPH_ERR_ARG;
  } else {
    rc = SPH_ERR_ARG;
  }
  if (v->sys) {
    DeviceGuard guard(v->sys->device);
    if (v->copy) cudaStreamSynchronize(v->copy);
    free_slots(v);
    for (int i = 0; i < kSlots; ++i) {
      if (v->gathered[i]) cudaEventDestroy(v->gathered[i]);
      if (v->copied[i]) cudaEventDestroy(v->copied[i]);
    }
    if (v->copy) cudaStreamDestroy(v->copy);
  }
  delete v;
  return rc;
}

int sph_vtk_frames(sph_vtk* v, int32_t* written) {
  if (!v || !written) return SPH_ERR_ARG;
  std::lock_guard<std::mutex> lk(v->mu);
  *written = (int32_t)v->written.size();
  return SPH_OK;
}

}  // extern "C"
