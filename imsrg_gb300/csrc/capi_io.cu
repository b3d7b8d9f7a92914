// extern "C" boundary, operator files (include/imsrg_gb300.h): a device
// operator (scalar or reduced tensor) written to / read from the reference's
// binary Operator layout
// (Operator::WriteBinary / ReadBinary, src/Operator.cc:341-388, with
// TwoBodyME::WriteBinary / ReadBinary, src/TwoBodyME.cc:812-836), so files
// interchange with IMSRG++.  The arena streams through two pinned staging
// buffers: the copy of one chunk overlaps the file I/O of the other.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "tensor.hpp"

using namespace imsrg;

namespace {

int ioerr(int code, const std::string& msg) { return set_error(code, msg.c_str()); }

constexpr size_t kChunk = (size_t)4 << 20;  // doubles per staging buffer (32 MiB)

// the arena pieces of a scalar operator in file order: ZeroBody, OneBody,
// then every two-body channel block (zero-size blocks write nothing)
struct Piece {
  int64_t off, len;
};

std::vector<Piece> pieces(const Space& s, const TensorLayout* t)
{
  std::vector<Piece> v;
  v.push_back({0, 1});
  v.push_back({32, (int64_t)s.norb * s.norb});
  if (t) {
    // a tensor's blocks in TwoBodyME::MatEl order (the layout's order)
    for (size_t b = 0; b < t->bra.size(); ++b) {
      int64_t n = (int64_t)s.ch[t->bra[b]].n() * s.ch[t->ket[b]].n();
      if (n) v.push_back({t->off[b], n});
    }
    return v;
  }
  for (int c = 0; c < s.nch; ++c) {
    int64_t n = s.ch[c].n();
    if (n) v.push_back({s.ch[c].off, n * n});
  }
  return v;
}

// Operator header, src/Operator.cc:341-352: rank_J, rank_T, parity,
// particle_rank, legs, E2max, E3max (int), hermitian, antihermitian (bool),
// nChannels (int)
#pragma pack(push, 1)
struct OpHeader {
  int32_t rank_J, rank_T, parity, particle_rank, legs, E2max, E3max;
  uint8_t hermitian, antihermitian;
  int32_t nChannels;
};
// TwoBodyME header, src/TwoBodyME.cc:812-818: nChannels (size_t), hermitian,
// antihermitian (bool), rank_J, rank_T, parity (int)
struct TbHeader {
  uint64_t nChannels;
  uint8_t hermitian, antihermitian;
  int32_t rank_J, rank_T, parity;
};
#pragma pack(pop)
static_assert(sizeof(OpHeader) == 34, "Operator header layout");
static_assert(sizeof(TbHeader) == 22, "TwoBodyME header layout");

struct Staging {
  double* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~Staging()
  {
    for (int i = 0; i < 2; ++i) {
      if (buf[i]) cudaFreeHost(buf[i]);
      if (ev[i]) cudaEventDestroy(ev[i]);
    }
  }
  int init()
  {
    for (int i = 0; i < 2; ++i) {
      if (cudaHostAlloc((void**)&buf[i], kChunk * sizeof(double), cudaHostAllocDefault) != cudaSuccess ||
          cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return ioerr(IMSRG_ERR_NOMEM, "pinned staging buffers");
      }
    }
    return IMSRG_OK;
  }
};

struct File {
  FILE* f = nullptr;
  ~File()
  {
    if (f) std::fclose(f);
  }
};

}  // namespace

extern "C" {

int imsrg_op_write_binary(const imsrg_op* op, const char* path, void* stream)
{
  if (!op || !path) return ioerr(IMSRG_ERR_ARG, "bad arguments");
  if (op->herm != 1 && op->herm != -1) return ioerr(IMSRG_ERR_UNSUPPORTED, "hermiticity must be +1 or -1");
  const Space& s = *op->sp->s;
  const TensorLayout* t = op->tl;
  const int rJ = t ? t->lam : 0, rT = t ? t->trank : 0, par = t ? t->parity : 0;
  cudaStream_t st = (cudaStream_t)stream;
  Staging stg;
  int rc = stg.init();
  if (rc) return rc;
  File fh;
  fh.f = std::fopen(path, "wb");
  if (!fh.f) return ioerr(IMSRG_ERR_IO, std::string("cannot open ") + path + " for writing");
  OpHeader oh{rJ, rT, par, 2, 4, 2 * s.emax, std::min(14, 3 * s.emax), (uint8_t)(op->herm == 1),
              (uint8_t)(op->herm == -1), s.nch};
  TbHeader th{(uint64_t)s.nch, oh.hermitian, oh.antihermitian, rJ, rT, par};
  if (std::fwrite(&oh, sizeof(oh), 1, fh.f) != 1) return ioerr(IMSRG_ERR_IO, "write failed");
  std::vector<Piece> pcs = pieces(s, t);
  // chunks of the arena [lo, hi) stream through the two staging buffers; the
  // pieces are in increasing arena order, so each chunk writes the parts of
  // the pieces it covers, in order
  const int64_t end = pcs.back().off + pcs.back().len;
  size_t ip = 0;
  int64_t done_in_piece = 0;
  auto flush = [&](int b, int64_t lo, int64_t hi) -> int {
    if (cudaEventSynchronize(stg.ev[b]) != cudaSuccess) return ioerr(IMSRG_ERR_CUDA, "device to host copy failed");
    while (ip < pcs.size()) {
      int64_t a = pcs[ip].off + done_in_piece, z = pcs[ip].off + pcs[ip].len;
      if (a >= hi) break;
      if (ip == 2 && done_in_piece == 0 && std::fwrite(&th, sizeof(th), 1, fh.f) != 1)
        return ioerr(IMSRG_ERR_IO, "write failed");
      int64_t w = std::min(z, hi) - a;
      if (w > 0 && std::fwrite(stg.buf[b] + (a - lo), sizeof(double), (size_t)w, fh.f) != (size_t)w)
        return ioerr(IMSRG_ERR_IO, "write failed");
      done_in_piece += w;
      if (done_in_piece == pcs[ip].len) {
        ++ip;
        done_in_piece = 0;
      }
    }
    return IMSRG_OK;
  };
  int64_t prev_lo = -1, prev_hi = -1;
  int k = 0;
  for (int64_t lo = 0; lo < end; lo += (int64_t)kChunk, ++k) {
    int64_t hi = std::min(end, lo + (int64_t)kChunk);
    int b = k & 1;
    if (cudaMemcpyAsync(stg.buf[b], op->d + lo, (hi - lo) * sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaEventRecord(stg.ev[b], st) != cudaSuccess)
      return ioerr(IMSRG_ERR_CUDA, "device to host copy failed");
    if (prev_lo >= 0 && (rc = flush(b ^ 1, prev_lo, prev_hi))) return rc;
    prev_lo = lo;
    prev_hi = hi;
  }
  if (prev_lo >= 0 && (rc = flush(k & 1 ? 0 : 1, prev_lo, prev_hi))) return rc;
  if (ip == 2 && std::fwrite(&th, sizeof(th), 1, fh.f) != 1) return ioerr(IMSRG_ERR_IO, "write failed");
  if (std::fflush(fh.f) != 0) return ioerr(IMSRG_ERR_IO, "write failed");
  return IMSRG_OK;
}

int imsrg_op_read_binary(imsrg_op* op, const char* path, void* stream)
{
  if (!op || !path) return ioerr(IMSRG_ERR_ARG, "bad arguments");
  const Space& s = *op->sp->s;
  const TensorLayout* t = op->tl;
  const int rJ = t ? t->lam : 0, rT = t ? t->trank : 0, par = t ? t->parity : 0;
  cudaStream_t st = (cudaStream_t)stream;
  File fh;
  fh.f = std::fopen(path, "rb");
  if (!fh.f) return ioerr(IMSRG_ERR_IO, std::string("cannot open ") + path);
  OpHeader oh;
  if (std::fread(&oh, sizeof(oh), 1, fh.f) != 1) return ioerr(IMSRG_ERR_IO, "file too short");
  if (oh.rank_J != rJ || oh.rank_T != rT || oh.parity != par)
    return ioerr(IMSRG_ERR_ARG, "the file's rank (J, T, parity) is not the operator's");
  if (oh.legs != 4 || oh.particle_rank != 2)
    return ioerr(IMSRG_ERR_UNSUPPORTED, "only two-body operators (legs = 4) are on the GPU path");
  if (oh.nChannels != s.nch) return ioerr(IMSRG_ERR_ARG, "file is for a model space with another channel count");
  int herm = oh.hermitian ? 1 : (oh.antihermitian ? -1 : 0);
  if (!herm) return ioerr(IMSRG_ERR_UNSUPPORTED, "operator is neither hermitian nor anti-hermitian");
  Staging stg;
  int rc = stg.init();
  if (rc) return rc;
  if (cudaMemsetAsync(op->d, 0, op->len * sizeof(double), st) != cudaSuccess)
    return ioerr(IMSRG_ERR_CUDA, "arena memset failed");
  std::vector<Piece> pcs = pieces(s, t);
  // file pieces fill a staging buffer; a full buffer goes to the device as one
  // copy per piece, and the other buffer fills meanwhile
  struct Pending {
    size_t boff;
    int64_t aoff, len;
  };
  std::vector<Pending> pend;
  int b = 0;
  size_t used = 0;
  bool inflight[2] = {false, false};
  auto submit = [&]() -> int {
    for (const Pending& p : pend)
      if (cudaMemcpyAsync(op->d + p.aoff, stg.buf[b] + p.boff, p.len * sizeof(double), cudaMemcpyHostToDevice,
                          st) != cudaSuccess)
        return ioerr(IMSRG_ERR_CUDA, "host to device copy failed");
    if (cudaEventRecord(stg.ev[b], st) != cudaSuccess) return ioerr(IMSRG_ERR_CUDA, "event record failed");
    inflight[b] = true;
    pend.clear();
    used = 0;
    b ^= 1;
    if (inflight[b] && cudaEventSynchronize(stg.ev[b]) != cudaSuccess)
      return ioerr(IMSRG_ERR_CUDA, "host to device copy failed");
    inflight[b] = false;
    return IMSRG_OK;
  };
  for (size_t ip = 0; ip < pcs.size(); ++ip) {
    if (ip == 2) {
      TbHeader th;
      if (std::fread(&th, sizeof(th), 1, fh.f) != 1) return ioerr(IMSRG_ERR_IO, "file too short");
      if (th.nChannels != (uint64_t)s.nch || th.rank_J != rJ || th.rank_T != rT || th.parity != par)
        return ioerr(IMSRG_ERR_ARG, "two-body header does not match the model space");
    }
    int64_t got = 0;
    while (got < pcs[ip].len) {
      if (used == kChunk && (rc = submit())) return rc;
      int64_t w = std::min<int64_t>(pcs[ip].len - got, (int64_t)(kChunk - used));
      if (std::fread(stg.buf[b] + used, sizeof(double), (size_t)w, fh.f) != (size_t)w)
        return ioerr(IMSRG_ERR_IO, "file too short for this model space");
      pend.push_back({used, pcs[ip].off + got, w});
      used += (size_t)w;
      got += w;
    }
  }
  if (pcs.size() == 2) {  // no two-body blocks: the header still follows
    TbHeader th;
    if (std::fread(&th, sizeof(th), 1, fh.f) != 1) return ioerr(IMSRG_ERR_IO, "file too short");
  }
  if (!pend.empty() && (rc = submit())) return rc;
  char extra;
  if (std::fread(&extra, 1, 1, fh.f) == 1) return ioerr(IMSRG_ERR_ARG, "file is longer than this model space's operator");
  if (cudaStreamSynchronize(st) != cudaSuccess) return ioerr(IMSRG_ERR_CUDA, "host to device copy failed");
  op->herm = herm;
  return IMSRG_OK;
}

}  // extern "C"
