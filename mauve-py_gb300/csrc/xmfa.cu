// XMFA writer: GenericIntervalList::WriteStandardAlignment
// (LM/IntervalList.h:353-440) for pairwise blocks, the file progressiveMauve
// writes and buildIndex parses.  The layout (which headers, their text, the
// 80-column rows, the "=" separators) is planned on the host; the text is
// assembled on the device in one kernel (header bytes from a staged blob,
// gapped rows wrapped at 80 columns straight from device memory) and copied
// out once.
//
// What the reference writes, for two sequences:
//   #FormatVersion Mauve1
//   #Sequence<i>File\t<name>          per sequence
//   #Sequence<i>Entry\t<i>            when both names are the same
//   #Sequence<i>Format\t<format>      by the name's extension (gnSourceFactory:
//                                     .fas/.FAS FastA, .seq/.SEQ DNAstar, .gbk/.GBK
//                                     /.gb/.GB GenBank, .raw/.RAW raw, else FastA),
//                                     DNAstar and GenBank with two #Annotation lines
//   #BackboneFile\t<name>             when a backbone file is named
//   per block with columns, per sequence (a sequence absent from a block,
//   start 0, is written only in the first block):
//   > <i>:<left>-<right> <+|-> <name> (0-0 + when absent; the first name for
//                                     both when the names are the same)
//   the row, 80 columns per line
//   =
#include <string.h>

#include <algorithm>

#include <string>
#include <vector>

#include "mvg_internal.h"

namespace mvg {

// A piece of the output: header bytes (src = offset in the staged blob) or a
// gapped row (src = its first column), at dst, len source bytes.
struct XmfaPiece {
  uint64_t dst, src, len;
  int32_t row;  // -1 header, 0 / 1 row of sequence A / B
  int32_t pad;
};

// Pieces along grid.y, each piece's output bytes spread over grid.x: output
// byte o of a row piece is column (o / 81) * 80 + o % 81 of the row, or the
// newline that ends every 80 columns and the last, partial line.
__global__ void k_xmfa_assemble(const XmfaPiece* __restrict__ pieces, int64_t npieces, const uint8_t* __restrict__ blob,
                                const uint8_t* __restrict__ rows_a, const uint8_t* __restrict__ rows_b,
                                uint8_t* __restrict__ out) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (int64_t k = blockIdx.y; k < npieces; k += gridDim.y) {
    const XmfaPiece pc = pieces[k];
    const uint64_t first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pc.row < 0) {
      for (uint64_t i = first; i < pc.len; i += step) out[pc.dst + i] = blob[pc.src + i];
    } else {
      const uint8_t* r = (pc.row == 0 ? rows_a : rows_b) + pc.src;
      const uint64_t nout = pc.len + (pc.len + 79) / 80;
      for (uint64_t o = first; o < nout; o += step) {
        const uint64_t line = o / 81, pos = o - line * 81, c = line * 80 + pos;
        out[pc.dst + o] = (pos == 80 || c == pc.len) ? (uint8_t)'\n' : r[c];
      }
    }
  }
}

static std::string format_of(const std::string& name) {
  const size_t dot = name.rfind('.');
  const std::string ext = dot == std::string::npos ? std::string() : name.substr(dot);
  if (ext == ".seq" || ext == ".SEQ") return "DNAstar";
  if (ext == ".gbk" || ext == ".GBK" || ext == ".gb" || ext == ".GB") return "GenBank";
  if (ext == ".raw" || ext == ".RAW") return "raw";
  return "FastA";  // .fas / .FAS and the default source class
}

static int xmfa_plan(const char* file_a, const char* file_b, const char* backbone, int64_t nblocks,
                     const int64_t* starts, const int64_t* lengths, const uint64_t* col_off, std::string* blob,
                     std::vector<XmfaPiece>* pieces, uint64_t* total) {
  const std::string names[2] = {file_a, file_b};
  const bool single = names[0] == names[1];
  blob->clear();
  pieces->clear();
  uint64_t dst = 0;
  auto header = [&](const std::string& s) {
    if (s.empty()) return;
    pieces->push_back(XmfaPiece{dst, (uint64_t)blob->size(), (uint64_t)s.size(), -1, 0});
    blob->append(s);
    dst += s.size();
  };
  if (nblocks == 0) {  // an empty list writes nothing
    *total = 0;
    return 0;
  }
  std::string h = "#FormatVersion Mauve1\n";
  for (int q = 0; q < 2; ++q) {
    const std::string i = std::to_string(q + 1);
    h += "#Sequence" + i + "File\t" + names[q] + "\n";
    if (single) h += "#Sequence" + i + "Entry\t" + i + "\n";
    const std::string f = format_of(names[q]);
    h += "#Sequence" + i + "Format\t" + f + "\n";
    if (f == "DNAstar" || f == "GenBank")
      h += "#Annotation" + i + "File\t" + names[q] + "\n#Annotation" + i + "Format\t" + f + "\n";
  }
  if (backbone && backbone[0]) h += std::string("#BackboneFile\t") + backbone + "\n";
  header(h);
  for (int64_t b = 0; b < nblocks; ++b) {
    if (col_off[b + 1] < col_off[b]) return report_error(MVG_ERR_ARG, "column offsets decrease");
    const uint64_t ncol = col_off[b + 1] - col_off[b];
    if (ncol == 0) continue;
    for (int q = 0; q < 2; ++q) {
      const int64_t s = starts[2 * b + q];
      const int64_t len = lengths[2 * b + q];
      if (s == 0 && b > 0) continue;  // the reference writes absent sequences into the first block only
      if (len < 0) return report_error(MVG_ERR_ARG, "negative block length");
      std::string line = "> " + std::to_string(q + 1) + ":";
      const uint64_t left = (uint64_t)(s < 0 ? -s : s);
      if (s == 0)
        line += "0-0 + ";
      else
        line += std::to_string(left) + "-" + std::to_string(left + (uint64_t)len - 1) + (s > 0 ? " + " : " - ");
      line += (single ? names[0] : names[q]) + "\n";
      header(line);
      pieces->push_back(XmfaPiece{dst, col_off[b], ncol, q, 0});
      dst += ncol + (ncol + 79) / 80;
    }
    header("=\n");
  }
  *total = dst;
  return 0;
}

}  // namespace mvg

using namespace mvg;

static Ctx* xmfa_ctx(mvg_handle h) { return reinterpret_cast<Ctx*>(h); }

extern "C" int mvg_xmfa_write_dev(mvg_handle h, const char* file_a, const char* file_b, const char* backbone_file,
                                  int64_t nblocks, const int64_t* starts, const int64_t* lengths,
                                  const uint8_t* d_rows_a, const uint8_t* d_rows_b, const uint64_t* col_off, char* out,
                                  uint64_t cap, uint64_t* out_len) {
  if (!h || !file_a || !file_b || !out_len || nblocks < 0 ||
      (nblocks && (!starts || !lengths || !col_off || !d_rows_a || !d_rows_b)) || (!out && cap))
    return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = xmfa_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  std::string blob;
  std::vector<XmfaPiece> pieces;
  uint64_t total = 0;
  if (int rc = xmfa_plan(file_a, file_b, backbone_file, nblocks, starts, lengths, col_off, &blob, &pieces, &total))
    return rc;
  *out_len = total;
  if (total > cap) return report_error(MVG_ERR_CAPACITY, "XMFA output buffer too small");
  if (total == 0) return 0;
  Workspace& ws = c->ws;
  XmfaPiece* d_pieces = (XmfaPiece*)ws.get(c, 70, pieces.size() * sizeof(XmfaPiece));
  uint8_t* d_blob = (uint8_t*)ws.get(c, 71, blob.size() + 16);
  uint8_t* d_out = (uint8_t*)ws.get(c, 72, total + 16);
  if (!d_pieces || !d_blob || !d_out) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (int rc = stage_reserve(c, pieces.size() * sizeof(XmfaPiece) + blob.size() + 1024)) return rc;
  if (int rc = h2d_async(c, d_pieces, pieces.data(), pieces.size() * sizeof(XmfaPiece), c->stream)) return rc;
  if (int rc = h2d_async(c, d_blob, blob.data(), blob.size(), c->stream)) return rc;
  const int64_t np = (int64_t)pieces.size();
  uint64_t widest = 0;  // output bytes of the largest piece
  for (const XmfaPiece& pc : pieces) widest = std::max(widest, pc.row < 0 ? pc.len : pc.len + (pc.len + 79) / 80);
  const dim3 grid((unsigned)std::min<uint64_t>(std::max<uint64_t>((widest + 1023) / 1024, 1), 1024),
                  (unsigned)std::min<int64_t>(np, 65535));
  k_xmfa_assemble<<<grid, 256, 0, c->stream>>>(d_pieces, np, d_blob, d_rows_a, d_rows_b, d_out);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  MVG_CUDA_TRY(cudaMemcpyAsync(out, d_out, total, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int mvg_xmfa_write(mvg_handle h, const char* file_a, const char* file_b, const char* backbone_file,
                              int64_t nblocks, const int64_t* starts, const int64_t* lengths, const uint8_t* rows_a,
                              const uint8_t* rows_b, const uint64_t* col_off, char* out, uint64_t cap,
                              uint64_t* out_len) {
  if (!h || nblocks < 0 || (nblocks && (!col_off || !rows_a || !rows_b)))
    return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = xmfa_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  const uint64_t ncols = nblocks ? col_off[nblocks] : 0;
  uint8_t* dra = (uint8_t*)c->ws.get(c, 68, ncols + 16);
  uint8_t* drb = (uint8_t*)c->ws.get(c, 69, ncols + 16);
  if (!dra || !drb) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (ncols) {
    MVG_CUDA_TRY(cudaMemcpyAsync(dra, rows_a, ncols, cudaMemcpyHostToDevice, c->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(drb, rows_b, ncols, cudaMemcpyHostToDevice, c->stream));
  }
  return mvg_xmfa_write_dev(h, file_a, file_b, backbone_file, nblocks, starts, lengths, dra, drb, col_off, out, cap,
                            out_len);
}
