// ingest.cu -- mesh ingest onto the device (the geometry entry points of
// include/j3dg.h).
//
// Binary PLY and STL: the header is parsed on the host, the body streams
// into device memory through two pinned chunks (the read of chunk k+1
// overlaps the copy of chunk k) and device kernels decode the records:
// each block stages 128 consecutive records in shared memory with aligned
// 16-byte loads, then one thread per record converts its fields (any PLY
// scalar type, either byte order) into float vertices, packed colours,
// normals and fan-triangulated index triples. Face records whose list
// lengths vary are located by a host walk and decoded by the same fields.
// Text formats are parsed on host threads (ingest_parse.cpp) and uploaded.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/j3dg.h"
#include "ingest_parse.h"
#include "internal.h"

using namespace j3dg::ingest;

namespace j3dg {
int ctx_fail(j3dg_ctx* c, int code, const std::string& msg);
}

namespace {

const int kRec = 128;                 // records per block
const uint32_t kStageBytes = 48 * 1024;
const size_t kChunk = 32u << 20;      // pinned chunk of the body stream
const int kMaxLists = 4;

struct Field {
  int8_t type = T_NONE;
  uint16_t off = 0;
};

struct VertexSpec {
  uint32_t stride = 0;
  uint8_t be = 0, has_n = 0, has_c = 0;
  Field xyz[3], nrm[3], rgb[3];
};

struct FaceSpec {
  uint32_t stride = 0;  // fixed layout only
  uint8_t be = 0;
  Field count;          // index-list count
  int8_t index_type = T_NONE;
  uint16_t index_off = 0;
  uint32_t n = 0;       // polygon size (fixed layout)
  uint8_t has_tc = 0;
  Field tc_count;
  int8_t tc_type = T_NONE;
  uint16_t tc_off = 0;
  uint32_t n_lists = 0;  // every list of the record, checked against the first record
  Field list_count[kMaxLists];
  uint32_t list_n[kMaxLists];
};

// ------------------------------------------------------------- device

__device__ __forceinline__ uint64_t ld_bytes(const uint8_t* p, int size, bool be) {
  uint64_t v = 0;
  for (int i = 0; i < size; ++i) v |= (uint64_t)p[be ? size - 1 - i : i] << (8 * i);
  return v;
}

__device__ __forceinline__ int dsize(int t) {
  return t == T_F64 ? 8 : (t == T_I32 || t == T_U32 || t == T_F32) ? 4 : (t == T_I16 || t == T_U16) ? 2 : 1;
}

__device__ float ld_float(const uint8_t* p, int t, bool be) {
  switch (t) {
    case T_F32: return __uint_as_float((uint32_t)ld_bytes(p, 4, be));
    case T_F64: return __double2float_rn(__longlong_as_double((long long)ld_bytes(p, 8, be)));
    case T_I8: return __int2float_rn((int8_t)p[0]);
    case T_U8: return __uint2float_rn(p[0]);
    case T_I16: return __int2float_rn((int16_t)ld_bytes(p, 2, be));
    case T_U16: return __uint2float_rn((uint16_t)ld_bytes(p, 2, be));
    case T_I32: return __int2float_rn((int32_t)ld_bytes(p, 4, be));
    case T_U32: return __uint2float_rn((uint32_t)ld_bytes(p, 4, be));
    default: return 0.f;
  }
}

__device__ int64_t ld_int(const uint8_t* p, int t, bool be) {
  switch (t) {
    case T_I8: return (int8_t)p[0];
    case T_U8: return p[0];
    case T_I16: return (int16_t)ld_bytes(p, 2, be);
    case T_U16: return (uint16_t)ld_bytes(p, 2, be);
    case T_I32: return (int32_t)ld_bytes(p, 4, be);
    case T_U32: return (uint32_t)ld_bytes(p, 4, be);
    default: return 0;
  }
}

// A colour channel: bytes as they are, other integers clamped to 0..255,
// floats scaled by 255, clamped and truncated (NaN -> 0).
__device__ uint32_t ld_channel(const uint8_t* p, int t, bool be) {
  if (t == T_F32 || t == T_F64) {
    float x = __fmul_rn(ld_float(p, t, be), 255.f);
    x = x < 0.f ? 0.f : (x > 255.f ? 255.f : x);
    return x == x ? (uint32_t)x : 0u;
  }
  const int64_t v = ld_int(p, t, be);
  return (uint32_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}

// Copies the bytes of records [r0, r0 + nrec) into shared memory with
// aligned 16-byte loads and returns the first record's address there. The
// source buffer is 256-byte aligned with at least 16 bytes of slack after
// its last record, so the rounded range stays inside the allocation.
__device__ const uint8_t* stage(const uint8_t* base, uint64_t r0, uint32_t nrec, uint32_t stride, uint8_t* sm,
                                bool use_sm) {
  const uint8_t* g0 = base + r0 * stride;
  if (!use_sm) return g0;
  const uintptr_t a0 = (uintptr_t)g0 & ~(uintptr_t)15;
  const uintptr_t a1 = ((uintptr_t)(g0 + (uint64_t)nrec * stride) + 15) & ~(uintptr_t)15;
  const uint4* src = reinterpret_cast<const uint4*>(a0);
  uint4* dst = reinterpret_cast<uint4*>(sm);
  const uint32_t n16 = (uint32_t)((a1 - a0) >> 4);
  for (uint32_t k = threadIdx.x; k < n16; k += blockDim.x) dst[k] = __ldg(src + k);
  __syncthreads();
  return sm + ((uintptr_t)g0 - a0);
}

__global__ void __launch_bounds__(kRec) k_ply_vertices(const uint8_t* base, uint64_t n, VertexSpec s, int use_sm,
                                                       float* V, uint32_t* C, float* N) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint64_t r0 = (uint64_t)blockIdx.x * kRec;
  const uint32_t nrec = (uint32_t)min((uint64_t)kRec, n - r0);
  const uint8_t* rec = stage(base, r0, nrec, s.stride, sm, use_sm != 0);
  if (threadIdx.x >= nrec) return;
  const uint8_t* p = rec + (uint64_t)threadIdx.x * s.stride;
  const uint64_t i = r0 + threadIdx.x;
  const bool be = s.be != 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) V[3 * i + k] = ld_float(p + s.xyz[k].off, s.xyz[k].type, be);
  if (s.has_n) {
#pragma unroll
    for (int k = 0; k < 3; ++k) N[3 * i + k] = ld_float(p + s.nrm[k].off, s.nrm[k].type, be);
  }
  if (s.has_c) {
    const uint32_t r = ld_channel(p + s.rgb[0].off, s.rgb[0].type, be);
    const uint32_t g = ld_channel(p + s.rgb[1].off, s.rgb[1].type, be);
    const uint32_t b = ld_channel(p + s.rgb[2].off, s.rgb[2].type, be);
    C[i] = 0xff000000u | (b << 16) | (g << 8) | r;
  }
}

// One face record: fan triangles (i0, i_k+1, i_k+2) at T[3 * tri_base ...]
// and, with a texcoord list of 2n values, their corner uv.
__device__ void emit_face(const uint8_t* idx, int itype, uint32_t cnt, const uint8_t* tc, int ttype, bool be,
                          uint64_t tri_base, uint32_t* T, float* UV) {
  if (cnt < 3) return;
  const int isz = dsize(itype);
  const uint32_t i0 = (uint32_t)ld_int(idx, itype, be);
  uint32_t prev = (uint32_t)ld_int(idx + isz, itype, be);
  for (uint32_t k = 0; k + 2 < cnt; ++k) {
    const uint32_t next = (uint32_t)ld_int(idx + (size_t)(k + 2) * isz, itype, be);
    const uint64_t t = tri_base + k;
    T[3 * t] = i0;
    T[3 * t + 1] = prev;
    T[3 * t + 2] = next;
    if (tc) {
      const int tsz = dsize(ttype);
      const uint32_t c[3] = {0, k + 1, k + 2};
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        UV[6 * t + 2 * j] = ld_float(tc + (size_t)(2 * c[j]) * tsz, ttype, be);
        UV[6 * t + 2 * j + 1] = ld_float(tc + (size_t)(2 * c[j] + 1) * tsz, ttype, be);
      }
    }
    prev = next;
  }
}

// Fixed layout: every record has the first record's list lengths (checked;
// a mismatch raises flag bit 1 and the host switches to the walked layout).
__global__ void __launch_bounds__(kRec) k_ply_faces(const uint8_t* base, uint64_t n, FaceSpec s, int use_sm,
                                                    uint32_t* T, float* UV, uint32_t* flag) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint64_t r0 = (uint64_t)blockIdx.x * kRec;
  const uint32_t nrec = (uint32_t)min((uint64_t)kRec, n - r0);
  const uint8_t* rec = stage(base, r0, nrec, s.stride, sm, use_sm != 0);
  if (threadIdx.x >= nrec) return;
  const uint8_t* p = rec + (uint64_t)threadIdx.x * s.stride;
  const uint64_t i = r0 + threadIdx.x;
  const bool be = s.be != 0;
  for (uint32_t k = 0; k < s.n_lists; ++k)
    if (ld_int(p + s.list_count[k].off, s.list_count[k].type, be) != (int64_t)s.list_n[k]) {
      atomicOr(flag, 1u);
      return;
    }
  const uint32_t per = s.n >= 3 ? s.n - 2 : 0;
  emit_face(p + s.index_off, s.index_type, s.n, s.has_tc ? p + s.tc_off : nullptr, s.tc_type, be, i * per, T, UV);
}

// Walked layout: the host located each record's index list (and texcoord
// list) and its first output triangle.
__global__ void k_ply_faces_walked(const uint8_t* base, uint64_t n, FaceSpec s, const uint64_t* list_off,
                                   const uint64_t* tc_off, const uint32_t* tri_base, uint32_t* T, float* UV,
                                   uint32_t* flag) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool be = s.be != 0;
  const uint8_t* p = base + list_off[i];
  const int64_t c = ld_int(p, s.count.type, be);
  if (c < 0) {
    atomicOr(flag, 4u);
    return;
  }
  const uint8_t* tc = nullptr;
  if (s.has_tc) {
    const uint8_t* q = base + tc_off[i];
    if (ld_int(q, s.tc_count.type, be) == 2 * c) tc = q + dsize(s.tc_count.type);
    else if (c >= 3) atomicOr(flag, 2u);
  }
  emit_face(p + dsize(s.count.type), s.index_type, (uint32_t)c, tc, s.tc_type, be, tri_base[i], T, UV);
}

// Binary STL (80-byte header, count, 50-byte records: normal, 3 vertices,
// attribute): triangle i -> vertices 3i..3i+2 (no welding).
__global__ void __launch_bounds__(kRec) k_stl(const uint8_t* base, uint64_t n, float* V, uint32_t* T) {
  __shared__ __align__(16) uint8_t sm[kRec * 50 + 32];
  const uint64_t r0 = (uint64_t)blockIdx.x * kRec;
  const uint32_t nrec = (uint32_t)min((uint64_t)kRec, n - r0);
  const uint8_t* rec = stage(base, r0, nrec, 50, sm, true);
  if (threadIdx.x >= nrec) return;
  const uint8_t* p = rec + (uint64_t)threadIdx.x * 50;
  const uint64_t i = r0 + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 9; ++k) V[9 * i + k] = __uint_as_float((uint32_t)ld_bytes(p + 12 + 4 * k, 4, false));
#pragma unroll
  for (int k = 0; k < 3; ++k) T[3 * i + k] = (uint32_t)(3 * i + k);
}

// mesh.cpp:216-228 convert_vertex_colors(uint32 -> float3)
__global__ void k_colors_to_float(const uint32_t* c, uint64_t n, float* out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = c[i];
  out[3 * i] = __fdiv_rn((float)(v & 255u), 255.f);
  out[3 * i + 1] = __fdiv_rn((float)((v >> 8) & 255u), 255.f);
  out[3 * i + 2] = __fdiv_rn((float)((v >> 16) & 255u), 255.f);
}

// ------------------------------------------------------------------ host

cudaStream_t S(j3dg_ctx* c) {
  ++c->stream_ops;
  return (cudaStream_t)c->stream;
}

int fail(j3dg_ctx* c, int code, const std::string& msg) { return j3dg::ctx_fail(c, code, msg); }

int cuda_fail(j3dg_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaErrorMemoryAllocation) return fail(c, J3DG_ERR_OUT_OF_MEMORY, std::string(where) + ": out of device memory");
  return fail(c, J3DG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CKG(x, where)                                  \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, where); \
  } while (0)

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Bytes of a file or of caller memory.
struct Source {
  int fd = -1;
  const uint8_t* mem = nullptr;
  uint64_t size = 0;
  double read_ms = 0;
  bool read(uint64_t off, void* dst, size_t len) {
    if (off > size || len > size - off) return false;
    if (mem) {
      memcpy(dst, mem + off, len);
      return true;
    }
    const double t0 = now_ms();
    uint8_t* d = (uint8_t*)dst;
    while (len) {
      const ssize_t r = pread(fd, d, len, (off_t)off);
      if (r <= 0) return false;
      d += r;
      off += (uint64_t)r;
      len -= (size_t)r;
    }
    read_ms += now_ms() - t0;
    return true;
  }
};

void free_geometry(j3dg_geometry* g) {
  cudaFree(g->d_v);
  cudaFree(g->d_t);
  cudaFree(g->d_c);
  cudaFree(g->d_n);
  cudaFree(g->d_uv);
  g->d_v = nullptr;
  g->d_t = nullptr;
  g->d_c = nullptr;
  g->d_n = nullptr;
  g->d_uv = nullptr;
}

template <class T>
int upload_vec(j3dg_ctx* c, const std::vector<T>& v, T** out, const char* what) {
  *out = nullptr;
  if (v.empty()) return J3DG_OK;
  CKG(cudaMalloc((void**)out, sizeof(T) * v.size()), what);
  CKG(cudaMemcpyAsync(*out, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, S(c)), what);
  return J3DG_OK;
}

int from_host(j3dg_ctx* c, HostGeometry& h, j3dg_geometry* g) {
  g->nv = h.vertices.size() / 3;
  g->nt = h.triangles.size() / 3;
  if (int rc = upload_vec(c, h.vertices, &g->d_v, "ingest upload")) return rc;
  if (int rc = upload_vec(c, h.triangles, &g->d_t, "ingest upload")) return rc;
  if (int rc = upload_vec(c, h.colors, &g->d_c, "ingest upload")) return rc;
  if (int rc = upload_vec(c, h.normals, &g->d_n, "ingest upload")) return rc;
  if (int rc = upload_vec(c, h.uv, &g->d_uv, "ingest upload")) return rc;
  g->info.has_colors = !h.colors.empty();
  g->info.has_normals = !h.normals.empty();
  g->info.has_uv = !h.uv.empty();
  CKG(cudaStreamSynchronize(S(c)), "ingest upload");
  return J3DG_OK;
}

// Streams src[off, off + len) into device memory at dst.
int stream_to_device(j3dg_ctx* c, Source& src, uint64_t off, uint64_t len, uint8_t* dst) {
  if (src.mem) {
    CKG(cudaMemcpyAsync(dst, src.mem + off, len, cudaMemcpyHostToDevice, S(c)), "ingest copy");
    return J3DG_OK;
  }
  void* stage[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int rc = J3DG_OK;
  cudaError_t e = cudaHostAlloc(&stage[0], kChunk, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaHostAlloc(&stage[1], kChunk, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  for (uint64_t at = 0, k = 0; e == cudaSuccess && rc == J3DG_OK && at < len; at += kChunk, ++k) {
    const size_t n = (size_t)std::min<uint64_t>(kChunk, len - at);
    const int b = (int)(k & 1);
    if (k >= 2) e = cudaEventSynchronize(ev[b]);
    if (e != cudaSuccess) break;
    if (!src.read(off + at, stage[b], n)) {
      rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: file read failed");
      break;
    }
    e = cudaMemcpyAsync(dst + at, stage[b], n, cudaMemcpyHostToDevice, S(c));
    if (e == cudaSuccess) e = cudaEventRecord(ev[b], S(c));
  }
  cudaError_t e2 = cudaStreamSynchronize(S(c));
  if (e == cudaSuccess) e = e2;
  for (int b = 0; b < 2; ++b) {
    if (ev[b]) cudaEventDestroy(ev[b]);
    if (stage[b]) cudaFreeHost(stage[b]);
  }
  if (rc == J3DG_OK && e != cudaSuccess) rc = cuda_fail(c, e, "ingest copy");
  return rc;
}

bool field_of(const PlyElement& e, const char* name, Field* f) {
  const int k = e.find(name);
  if (k < 0 || e.props[k].list) return false;
  uint32_t off = 0;
  for (int j = 0; j < k; ++j) off += (uint32_t)type_size(e.props[j].type);
  f->type = e.props[k].type;
  f->off = (uint16_t)off;
  return true;
}

uint32_t stage_smem(uint32_t stride) {
  const uint32_t b = ((uint32_t)kRec * stride + 32 + 15) & ~15u;
  return b <= kStageBytes ? b : 0;
}

int read_ply_binary(j3dg_ctx* c, Source& src, const PlyHeader& h, j3dg_geometry* g) {
  const bool be = h.encoding == 2;
  int ev = -1, ef = -1;
  for (int i = 0; i < (int)h.elements.size(); ++i) {
    if (h.elements[i].name == "vertex" && ev < 0) ev = i;
    if (h.elements[i].name == "face" && ef < 0) ef = i;
  }
  if (ev < 0) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: no vertex element");
  const PlyElement& E = h.elements[ev];
  if (E.has_list()) return fail(c, J3DG_ERR_UNSUPPORTED, "ply: list property in the vertex element");
  VertexSpec vs;
  vs.stride = E.fixed_size();
  vs.be = be;
  if (!field_of(E, "x", &vs.xyz[0]) || !field_of(E, "y", &vs.xyz[1]) || !field_of(E, "z", &vs.xyz[2]))
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: vertex element without x, y, z");
  vs.has_n = field_of(E, "nx", &vs.nrm[0]) && field_of(E, "ny", &vs.nrm[1]) && field_of(E, "nz", &vs.nrm[2]);
  vs.has_c = field_of(E, "red", &vs.rgb[0]) && field_of(E, "green", &vs.rgb[1]) && field_of(E, "blue", &vs.rgb[2]);
  if (vs.stride > 65535) return fail(c, J3DG_ERR_UNSUPPORTED, "ply: vertex record larger than 64 KB");

  const uint64_t body = h.header_bytes, body_len = src.size - body;
  // element offsets up to the last one needed (list elements walked on the host)
  const int last = std::max(ev, ef);
  std::vector<uint64_t> off(h.elements.size() + 1, 0);
  std::vector<uint8_t> host_body;  // read on demand for walks
  auto host_bytes = [&]() -> bool {
    if (!host_body.empty() || body_len == 0) return true;
    host_body.resize(body_len);
    return src.read(body, host_body.data(), body_len);
  };
  for (int i = 0; i < last; ++i) {
    const PlyElement& e = h.elements[i];
    const uint32_t fs = e.fixed_size();
    if (fs) {
      if (e.count > (body_len - std::min(body_len, off[i])) / fs)
        return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: body shorter than the header says");
      off[i + 1] = off[i] + e.count * fs;
    } else {
      if (!host_bytes()) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: file read failed");
      size_t end = 0;
      if (!skip_binary_element(host_body.data(), host_body.size(), off[i], e, be, &end))
        return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: body shorter than the header says");
      off[i + 1] = end;
    }
  }
  const uint64_t v_off = off[ev];
  if (E.count > (body_len - std::min(body_len, v_off)) / std::max<uint32_t>(1, vs.stride))
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: body shorter than the header says");

  // face layout from the first record
  FaceSpec fsx;
  fsx.be = be;
  bool fixed = true;
  uint64_t n_faces = 0, n_tris = 0, f_off = 0;
  int il = -1, itc = -1;
  if (ef >= 0 && h.elements[ef].count > 0) {
    const PlyElement& F = h.elements[ef];
    n_faces = F.count;
    f_off = off[ef];
    il = F.find("vertex_indices");
    if (il < 0) il = F.find("vertex_index");
    itc = F.find("texcoord");
    if (itc < 0) itc = F.find("texcoords");
    if (il < 0 || !F.props[il].list) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: face element without a vertex_indices list");
    if (F.props[il].item_type == T_F32 || F.props[il].item_type == T_F64)
      return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: vertex_indices must be integers");
    if (itc >= 0 && !F.props[itc].list) itc = -1;
    fsx.count.type = F.props[il].count_type;
    fsx.index_type = F.props[il].item_type;
    if (itc >= 0) {
      fsx.has_tc = 1;
      fsx.tc_count.type = F.props[itc].count_type;
      fsx.tc_type = F.props[itc].item_type;
    }
    // first record
    uint8_t first[4096];
    const size_t avail = (size_t)std::min<uint64_t>(sizeof(first), body_len - std::min(body_len, f_off));
    if (!src.read(body + f_off, first, avail)) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: file read failed");
    uint32_t at = 0;
    int lists = 0;
    for (int k = 0; k < (int)F.props.size() && fixed; ++k) {
      const PlyProp& pr = F.props[k];
      if (!pr.list) {
        at += type_size(pr.type);
        continue;
      }
      const int cs = type_size(pr.count_type);
      if (at + cs > avail) {
        fixed = false;
        break;
      }
      uint64_t raw = 0;
      for (int b = 0; b < cs; ++b) raw |= (uint64_t)first[at + (be ? cs - 1 - b : b)] << (8 * b);
      int64_t cnt = (pr.count_type == T_I8) ? (int8_t)raw : (pr.count_type == T_I16) ? (int16_t)raw
                    : (pr.count_type == T_I32) ? (int32_t)raw : (int64_t)raw;
      if (cnt < 0 || lists >= kMaxLists || cnt > 4096) {
        fixed = false;
        break;
      }
      fsx.list_count[lists].type = pr.count_type;
      fsx.list_count[lists].off = (uint16_t)at;
      fsx.list_n[lists] = (uint32_t)cnt;
      ++lists;
      if (k == il) {
        fsx.count.off = (uint16_t)at;
        fsx.index_off = (uint16_t)(at + cs);
        fsx.n = (uint32_t)cnt;
      }
      if (k == itc) {
        fsx.tc_count.off = (uint16_t)at;
        fsx.tc_off = (uint16_t)(at + cs);
        if (cnt != 2 * (int64_t)fsx.n) fsx.has_tc = 0;  // uv only with 2 values per corner
      }
      at += cs + (uint32_t)cnt * type_size(pr.item_type);
      if (at > 60000) {
        fixed = false;
        break;
      }
    }
    fsx.n_lists = (uint32_t)lists;
    fsx.stride = at;
    if (fixed && (fsx.stride == 0 || n_faces > (body_len - std::min(body_len, f_off)) / fsx.stride)) fixed = false;
    if (fixed) n_tris = n_faces * (fsx.n >= 3 ? fsx.n - 2 : 0);
  }

  // body -> device
  uint8_t* d_body = nullptr;
  uint32_t* d_flag = nullptr;
  int rc = J3DG_OK;
  CKG(cudaMalloc(&d_body, body_len + 64), "ingest body");
  auto done = [&](int code) {
    cudaStreamSynchronize(S(c));
    cudaFree(d_body);
    cudaFree(d_flag);
    return code;
  };
  if ((rc = stream_to_device(c, src, body, body_len, d_body))) return done(rc);
  cudaError_t e = cudaMalloc((void**)&d_flag, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(uint32_t), S(c));
  g->nv = E.count;
  if (e == cudaSuccess && g->nv) e = cudaMalloc((void**)&g->d_v, sizeof(float) * 3 * g->nv);
  if (e == cudaSuccess && g->nv && vs.has_c) e = cudaMalloc((void**)&g->d_c, sizeof(uint32_t) * g->nv);
  if (e == cudaSuccess && g->nv && vs.has_n) e = cudaMalloc((void**)&g->d_n, sizeof(float) * 3 * g->nv);
  if (e == cudaSuccess && g->nv) {
    const uint32_t smem = stage_smem(vs.stride);
    const uint64_t blocks = (g->nv + kRec - 1) / kRec;
    k_ply_vertices<<<(unsigned)blocks, kRec, smem, S(c)>>>(d_body + v_off, g->nv, vs, smem ? 1 : 0, g->d_v, g->d_c,
                                                          g->d_n);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return done(cuda_fail(c, e, "ingest vertices"));
  g->info.has_colors = vs.has_c;
  g->info.has_normals = vs.has_n;

  if (n_faces) {
    uint32_t flag = 0;
    if (fixed) {
      g->nt = n_tris;
      if (n_tris >= 0xffffffffull) return done(fail(c, J3DG_ERR_UNSUPPORTED, "ply: more than 2^32 triangles"));
      if (n_tris) e = cudaMalloc((void**)&g->d_t, sizeof(uint32_t) * 3 * n_tris);
      if (e == cudaSuccess && n_tris && fsx.has_tc) e = cudaMalloc((void**)&g->d_uv, sizeof(float) * 6 * n_tris);
      if (e == cudaSuccess) {  // also when the first face has < 3 corners: the launch checks the layout
        const uint32_t smem = stage_smem(fsx.stride);
        k_ply_faces<<<(unsigned)((n_faces + kRec - 1) / kRec), kRec, smem, S(c)>>>(
            d_body + f_off, n_faces, fsx, smem ? 1 : 0, g->d_t, g->d_uv, d_flag);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, S(c));
      if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));
      if (e != cudaSuccess) return done(cuda_fail(c, e, "ingest faces"));
      if (flag & 1) {  // lists vary: walked layout
        fixed = false;
        cudaFree(g->d_t);
        cudaFree(g->d_uv);
        g->d_t = nullptr;
        g->d_uv = nullptr;
      }
    }
    if (!fixed) {
      if (!host_bytes()) return done(fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: file read failed"));
      std::vector<uint64_t> list_off, tc_off;
      std::vector<uint32_t> tri_base;
      size_t end = 0;
      std::string err;
      if (!walk_binary_faces(host_body.data(), host_body.size(), f_off, h.elements[ef], be, il, itc, list_off, tc_off,
                             tri_base, &n_tris, &end, err))
        return done(fail(c, J3DG_ERR_INVALID_ARGUMENT, err));
      g->nt = n_tris;
      fsx.has_tc = itc >= 0;
      uint64_t* d_lo = nullptr;
      uint64_t* d_to = nullptr;
      uint32_t* d_tb = nullptr;
      e = cudaMemsetAsync(d_flag, 0, sizeof(uint32_t), S(c));
      if (e == cudaSuccess && n_tris) e = cudaMalloc((void**)&g->d_t, sizeof(uint32_t) * 3 * n_tris);
      if (e == cudaSuccess && n_tris && fsx.has_tc) e = cudaMalloc((void**)&g->d_uv, sizeof(float) * 6 * n_tris);
      if (e == cudaSuccess) e = cudaMalloc((void**)&d_lo, sizeof(uint64_t) * n_faces);
      if (e == cudaSuccess && fsx.has_tc) e = cudaMalloc((void**)&d_to, sizeof(uint64_t) * n_faces);
      if (e == cudaSuccess) e = cudaMalloc((void**)&d_tb, sizeof(uint32_t) * n_faces);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_lo, list_off.data(), sizeof(uint64_t) * n_faces, cudaMemcpyHostToDevice, S(c));
      if (e == cudaSuccess && fsx.has_tc)
        e = cudaMemcpyAsync(d_to, tc_off.data(), sizeof(uint64_t) * n_faces, cudaMemcpyHostToDevice, S(c));
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_tb, tri_base.data(), sizeof(uint32_t) * n_faces, cudaMemcpyHostToDevice, S(c));
      if (e == cudaSuccess && n_tris) {
        k_ply_faces_walked<<<(unsigned)((n_faces + 255) / 256), 256, 0, S(c)>>>(d_body, n_faces, fsx, d_lo, d_to, d_tb,
                                                                               g->d_t, g->d_uv, d_flag);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, S(c));
      if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));
      cudaFree(d_lo);
      cudaFree(d_to);
      cudaFree(d_tb);
      if (e != cudaSuccess) return done(cuda_fail(c, e, "ingest faces"));
      if (flag & 4) return done(fail(c, J3DG_ERR_INVALID_ARGUMENT, "ply: bad list count"));
    }
    if (flag & 2) {  // some faces without 2 texcoords per corner: no uv
      cudaFree(g->d_uv);
      g->d_uv = nullptr;
    }
    g->info.has_uv = g->d_uv != nullptr;
  }
  e = cudaStreamSynchronize(S(c));
  if (e != cudaSuccess) return done(cuda_fail(c, e, "ingest decode"));
  g->info.device_decoded = 1;
  return done(J3DG_OK);
}

int read_stl_binary(j3dg_ctx* c, Source& src, uint64_t n, j3dg_geometry* g) {
  uint8_t* d_body = nullptr;
  CKG(cudaMalloc(&d_body, 50 * n + 64), "ingest body");
  int rc = stream_to_device(c, src, 84, 50 * n, d_body);
  cudaError_t e = cudaSuccess;
  if (rc == J3DG_OK) {
    g->nv = 3 * n;
    g->nt = n;
    e = cudaMalloc((void**)&g->d_v, sizeof(float) * 9 * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&g->d_t, sizeof(uint32_t) * 3 * n);
    if (e == cudaSuccess) {
      k_stl<<<(unsigned)((n + kRec - 1) / kRec), kRec, 0, S(c)>>>(d_body, n, g->d_v, g->d_t);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));
    if (e != cudaSuccess) rc = cuda_fail(c, e, "ingest stl");
  }
  cudaStreamSynchronize(S(c));
  cudaFree(d_body);
  g->info.device_decoded = rc == J3DG_OK;
  return rc;
}

int format_of_path(const char* path) {
  const char* dot = strrchr(path, '.');
  const char* slash = strrchr(path, '/');
  if (!dot || (slash && dot < slash)) return J3DG_FORMAT_AUTO;
  std::string ext(dot + 1);
  for (auto& ch : ext) ch = (char)tolower((unsigned char)ch);
  if (ext == "ply") return J3DG_FORMAT_PLY;
  if (ext == "stl") return J3DG_FORMAT_STL;
  if (ext == "obj") return J3DG_FORMAT_OBJ;
  if (ext == "off") return J3DG_FORMAT_OFF;
  if (ext == "xyz") return J3DG_FORMAT_XYZ;
  if (ext == "pts") return J3DG_FORMAT_PTS;
  return J3DG_FORMAT_AUTO;
}

int read_any(j3dg_ctx* c, Source& src, int format, j3dg_geometry** out) {
  const double t0 = now_ms();
  j3dg_geometry* g = new (std::nothrow) j3dg_geometry();
  if (!g) return J3DG_ERR_OUT_OF_MEMORY;
  memset(&g->info, 0, sizeof(g->info));
  g->ctx = c;
  g->hold.attach(c);
  g->info.file_bytes = src.size;
  // header bytes for format detection and the PLY / STL headers
  std::vector<char> head((size_t)std::min<uint64_t>(src.size, 1 << 16));
  int rc = J3DG_OK;
  if (!src.read(0, head.data(), head.size())) rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: read failed");
  if (rc == J3DG_OK && format == J3DG_FORMAT_AUTO) {
    if (head.size() >= 3 && memcmp(head.data(), "ply", 3) == 0) format = J3DG_FORMAT_PLY;
    else if (head.size() >= 3 && (memcmp(head.data(), "OFF", 3) == 0 || (head.size() >= 4 && memcmp(head.data(), "COFF", 4) == 0)))
      format = J3DG_FORMAT_OFF;
    else if (head.size() >= 84) {
      uint32_t n;
      memcpy(&n, head.data() + 80, 4);
      if (src.size == 84 + 50ull * n) format = J3DG_FORMAT_STL;
    }
    if (format == J3DG_FORMAT_AUTO && head.size() >= 5 && memcmp(head.data(), "solid", 5) == 0) format = J3DG_FORMAT_STL;
    if (format == J3DG_FORMAT_AUTO) rc = fail(c, J3DG_ERR_UNSUPPORTED, "ingest: unknown file format");
  }
  g->info.format = (uint32_t)format;
  std::string err;
  HostGeometry hg;
  auto whole = [&](std::vector<char>& buf) -> bool {
    buf.resize(src.size);
    return src.size == 0 || src.read(0, buf.data(), src.size);
  };
  std::vector<char> buf;
  if (rc == J3DG_OK) {
    switch (format) {
      case J3DG_FORMAT_PLY: {
        PlyHeader h;
        bool ok = parse_ply_header(head.data(), head.size(), h, err);
        if (!ok && err.empty() && src.size > head.size()) {  // long header
          if (!whole(buf)) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: read failed"); break; }
          ok = parse_ply_header(buf.data(), buf.size(), h, err);
        }
        if (!ok) {
          rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, err.empty() ? "ply: header without end_header" : err);
          break;
        }
        g->info.encoding = (uint32_t)h.encoding;
        if (h.encoding == 0) {
          if (buf.empty() && !whole(buf)) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: read failed"); break; }
          if (!parse_ply_ascii(buf.data() + h.header_bytes, buf.size() - h.header_bytes, h, hg, err)) {
            rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, err);
            break;
          }
          rc = from_host(c, hg, g);
        } else {
          buf.clear();
          buf.shrink_to_fit();
          rc = read_ply_binary(c, src, h, g);
        }
        break;
      }
      case J3DG_FORMAT_STL: {
        uint32_t n = 0;
        if (head.size() >= 84) memcpy(&n, head.data() + 80, 4);
        if (head.size() >= 84 && src.size == 84 + 50ull * n) {
          g->info.encoding = 1;
          rc = n ? read_stl_binary(c, src, n, g) : J3DG_OK;
        } else {
          if (!whole(buf)) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: read failed"); break; }
          if (!parse_stl_ascii(buf.data(), buf.size(), hg, err)) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, err); break; }
          rc = from_host(c, hg, g);
        }
        break;
      }
      case J3DG_FORMAT_OBJ:
      case J3DG_FORMAT_OFF:
      case J3DG_FORMAT_XYZ:
      case J3DG_FORMAT_PTS: {
        if (!whole(buf)) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: read failed"); break; }
        bool ok = false;
        const int threads = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        if (format == J3DG_FORMAT_OBJ) ok = parse_obj(buf.data(), buf.size(), threads, hg, err);
        if (format == J3DG_FORMAT_OFF) ok = parse_off(buf.data(), buf.size(), hg, err);
        if (format == J3DG_FORMAT_XYZ) ok = parse_xyz(buf.data(), buf.size(), hg, err);
        if (format == J3DG_FORMAT_PTS) ok = parse_pts(buf.data(), buf.size(), hg, err);
        if (!ok) { rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, err); break; }
        rc = from_host(c, hg, g);
        break;
      }
      default:
        rc = fail(c, J3DG_ERR_UNSUPPORTED, "ingest: unknown file format");
    }
  }
  if (rc == J3DG_OK && g->nv == 0) rc = fail(c, J3DG_ERR_INVALID_ARGUMENT, "ingest: no vertices");
  if (rc == J3DG_OK && (g->nv >= 0xffffffffull || g->nt >= 0xffffffffull))
    rc = fail(c, J3DG_ERR_UNSUPPORTED, "ingest: more than 2^32 vertices or triangles");
  if (rc != J3DG_OK) {
    free_geometry(g);
    delete g;
    return rc;
  }
  g->info.n_vertices = g->nv;
  g->info.n_triangles = g->nt;
  g->info.read_ms = (float)src.read_ms;
  g->info.total_ms = (float)(now_ms() - t0);
  g->info.decode_ms = g->info.total_ms - g->info.read_ms;
  *out = g;
  return J3DG_OK;
}

}  // namespace

extern "C" {

int j3dg_geometry_read_file(j3dg_ctx* c, const char* path, int format, j3dg_geometry** out) {
  if (!c || !path || !out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (format < J3DG_FORMAT_AUTO || format > J3DG_FORMAT_PTS) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "bad format");
  if (format == J3DG_FORMAT_AUTO) format = format_of_path(path);
  if (format == J3DG_FORMAT_AUTO) return fail(c, J3DG_ERR_UNSUPPORTED, std::string("ingest: unknown extension: ") + path);
  cudaSetDevice(c->device);
  Source src;
  src.fd = open(path, O_RDONLY);
  if (src.fd < 0) return fail(c, J3DG_ERR_INVALID_ARGUMENT, std::string("ingest: cannot open ") + path);
  struct stat st;
  if (fstat(src.fd, &st) != 0) {
    close(src.fd);
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, std::string("ingest: cannot stat ") + path);
  }
  src.size = (uint64_t)st.st_size;
  const int rc = read_any(c, src, format, out);
  close(src.fd);
  return rc;
}

int j3dg_geometry_read_memory(j3dg_ctx* c, const void* bytes, uint64_t n, int format, j3dg_geometry** out) {
  if (!c || (!bytes && n) || !out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (format < J3DG_FORMAT_AUTO || format > J3DG_FORMAT_PTS) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "bad format");
  cudaSetDevice(c->device);
  Source src;
  src.mem = (const uint8_t*)bytes;
  src.size = n;
  return read_any(c, src, format, out);
}

int j3dg_geometry_get_info(const j3dg_geometry* g, j3dg_geometry_info* info) {
  if (!g || !info) return J3DG_ERR_INVALID_ARGUMENT;
  *info = g->info;
  return J3DG_OK;
}

int j3dg_geometry_get_arrays(const j3dg_geometry* g, float* V, uint32_t* T, uint32_t* C, float* N, float* UV) {
  if (!g) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = g->ctx;
  cudaSetDevice(c->device);
  if ((C && !g->d_c) || (N && !g->d_n) || (UV && !g->d_uv))
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, "geometry_get_arrays: the geometry has no such array");
  auto copy = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!dst || !bytes) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, S(c));
  };
  CKG(copy(V, g->d_v, sizeof(float) * 3 * g->nv), "geometry_get_arrays");
  CKG(copy(T, g->d_t, sizeof(uint32_t) * 3 * g->nt), "geometry_get_arrays");
  CKG(copy(C, g->d_c, sizeof(uint32_t) * g->nv), "geometry_get_arrays");
  CKG(copy(N, g->d_n, sizeof(float) * 3 * g->nv), "geometry_get_arrays");
  CKG(copy(UV, g->d_uv, sizeof(float) * 6 * g->nt), "geometry_get_arrays");
  CKG(cudaStreamSynchronize(S(c)), "geometry_get_arrays");
  return J3DG_OK;
}

int j3dg_geometry_destroy(j3dg_geometry* g) {
  if (!g) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(g->ctx->device);
  cudaStreamSynchronize(S(g->ctx));
  free_geometry(g);
  delete g;
  return J3DG_OK;
}

int j3dg_mesh_build_geometry(j3dg_ctx* c, const j3dg_geometry* g, const j3dg_build_opts* opts, j3dg_mesh** out) {
  if (!c || !g || !out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (g->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "mesh_build_geometry: geometry of another context");
  if (g->nt == 0) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "mesh_build_geometry: no triangles (a point cloud)");
  j3dg_mesh* m = nullptr;
  int rc = j3dg_mesh_build(c, g->d_v, (uint32_t)g->nv, g->d_t, (uint32_t)g->nt, opts, &m);
  if (rc != J3DG_OK) return rc;
  cudaError_t e = cudaSuccess;
  if (g->d_c) {
    e = cudaMalloc(&m->d_colors, sizeof(float) * 3 * g->nv);
    if (e == cudaSuccess) {
      k_colors_to_float<<<(unsigned)((g->nv + 255) / 256), 256, 0, S(c)>>>(g->d_c, g->nv, (float*)m->d_colors);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess && g->d_uv) {
    e = cudaMalloc(&m->d_uv, sizeof(float) * 6 * g->nt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_uv, g->d_uv, sizeof(float) * 6 * g->nt, cudaMemcpyDeviceToDevice, S(c));
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));
  if (e != cudaSuccess) {
    j3dg_mesh_destroy(m);
    return cuda_fail(c, e, "mesh_build_geometry");
  }
  if (g->d_uv) {  // mesh.cpp:172-173
    const std::vector<uint32_t> tex = dummy_texture(512, 512, 32);
    rc = j3dg_mesh_set_texture(m, tex.data(), 512, 512);
    if (rc != J3DG_OK) {
      j3dg_mesh_destroy(m);
      return rc;
    }
  }
  *out = m;
  return J3DG_OK;
}

}  // extern "C"
