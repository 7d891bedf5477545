// The reference's text formats, read on the host into the device graph:
//   vertex file  one oid per line (the .v file)
//   edge file    "u v" or "u v w" per line, oids (the .e file; weights are
//                the SSSP edge data, ignored for unweighted loads)
//   update file  "a u v [w]" inserts, "d u v" deletes
//                (grape/fragment/inc_fragment_builder.h:38-70)
//   cluster file records "size oid_1 ... oid_size" (the <efile>.c_<k> file
//                read by compress_by_cluster, compressor_base.h:3174-3243)
// Vertex ids are the ranks of the distinct oids (the vertex map of
// grape/vertex_map/global_vertex_map.h:145-166: oids 0..N-1 keep their
// value).  Lines starting with '#' are comments.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

namespace sg {

namespace {

struct FileBuf {
  std::vector<char> data;
  bool ok = false;
};

FileBuf read_all(const char* path) {
  FileBuf b;
  FILE* f = std::fopen(path, "rb");
  if (!f) return b;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    return b;
  }
  b.data.resize((size_t)sz + 1);
  const size_t got = sz > 0 ? std::fread(b.data.data(), 1, (size_t)sz, f) : 0;
  std::fclose(f);
  b.data[got] = '\0';
  b.data.resize(got + 1);
  b.ok = true;
  return b;
}

// Cursor over one text buffer: numbers, words, line ends.
struct Cursor {
  const char* p;
  const char* end;
  bool at_end() {
    skip_blank();
    return p >= end || *p == '\0';
  }
  void skip_blank() {
    for (;;) {
      while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
      if (p < end && *p == '#') {
        while (p < end && *p != '\n' && *p != '\0') ++p;
        continue;
      }
      break;
    }
  }
  void skip_spaces() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  }
  bool line_has_more() {
    skip_spaces();
    return p < end && *p != '\n' && *p != '\0' && *p != '#';
  }
  void next_line() {
    while (p < end && *p != '\n' && *p != '\0') ++p;
  }
  bool read_u64(uint64_t* out) {
    skip_spaces();
    if (p >= end || *p < '0' || *p > '9') return false;
    uint64_t v = 0;
    while (p < end && *p >= '0' && *p <= '9') v = v * 10 + (uint64_t)(*p++ - '0');
    *out = v;
    return true;
  }
  bool read_f64(double* out) {
    skip_spaces();
    char* e = nullptr;
    const double v = std::strtod(p, &e);
    if (e == p) return false;
    p = e;
    *out = v;
    return true;
  }
};

Cursor cursor(const FileBuf& b) { return Cursor{b.data.data(), b.data.data() + b.data.size() - 1}; }

}  // namespace

// oid -> vid by binary search over the sorted distinct oids (identity when
// the oids are exactly 0..n-1)
static bool oid_to_vid(const sg_ctx* ctx, uint64_t oid, uint32_t* vid) {
  const std::vector<uint64_t>& o = ctx->oids;
  if (o.empty()) {
    if (oid >= ctx->g.n) return false;
    *vid = (uint32_t)oid;
    return true;
  }
  auto it = std::lower_bound(o.begin(), o.end(), oid);
  if (it == o.end() || *it != oid) return false;
  *vid = (uint32_t)(it - o.begin());
  return true;
}

sg_status load_files(sg_ctx* ctx, const char* efile, const char* vfile, bool weighted) {
  FileBuf eb = read_all(efile);
  if (!eb.ok) return fail(ctx, SG_ERR_INVALID, std::string("cannot read edge file ") + efile);
  std::vector<uint64_t> src, dst;
  std::vector<float> wt;
  Cursor c = cursor(eb);
  while (!c.at_end()) {
    uint64_t u, v;
    if (!c.read_u64(&u) || !c.read_u64(&v))
      return fail(ctx, SG_ERR_INVALID, std::string("malformed edge line in ") + efile);
    double w = 1.0;
    if (c.line_has_more() && !c.read_f64(&w))
      return fail(ctx, SG_ERR_INVALID, std::string("malformed edge weight in ") + efile);
    src.push_back(u);
    dst.push_back(v);
    if (weighted) wt.push_back((float)w);
    c.next_line();
  }
  std::vector<uint64_t> oids;
  if (vfile && *vfile) {
    FileBuf vb = read_all(vfile);
    if (!vb.ok) return fail(ctx, SG_ERR_INVALID, std::string("cannot read vertex file ") + vfile);
    Cursor cv = cursor(vb);
    while (!cv.at_end()) {
      uint64_t o;
      if (!cv.read_u64(&o))
        return fail(ctx, SG_ERR_INVALID, std::string("malformed vertex line in ") + vfile);
      oids.push_back(o);
      cv.next_line();
    }
  } else {
    oids = src;
    oids.insert(oids.end(), dst.begin(), dst.end());
  }
  std::sort(oids.begin(), oids.end());
  oids.erase(std::unique(oids.begin(), oids.end()), oids.end());
  if (oids.empty()) return fail(ctx, SG_ERR_INVALID, "no vertices");
  if (oids.size() > 0xFFFFFFFEull) return fail(ctx, SG_ERR_INVALID, "too many vertices");
  const uint32_t n = (uint32_t)oids.size();
  const bool identity = oids.front() == 0 && oids.back() == (uint64_t)n - 1;
  ctx->oids.clear();
  if (!identity) ctx->oids = oids;
  ctx->g.n = n;  // for oid_to_vid during the mapping below
  std::vector<uint64_t> rp((size_t)n + 1, 0);
  std::vector<uint32_t> su(src.size()), dv(src.size());
  for (size_t i = 0; i < src.size(); ++i) {
    if (!oid_to_vid(ctx, src[i], &su[i]) || !oid_to_vid(ctx, dst[i], &dv[i]))
      return fail(ctx, SG_ERR_INVALID, "edge endpoint missing from the vertex file");
    rp[su[i] + 1]++;
  }
  for (uint32_t v = 0; v < n; ++v) rp[v + 1] += rp[v];
  std::vector<uint32_t> col(src.size());
  std::vector<float> w(weighted ? src.size() : 0);
  std::vector<uint64_t> pos(rp.begin(), rp.end() - 1);
  for (size_t i = 0; i < src.size(); ++i) {
    const uint64_t p = pos[su[i]]++;
    col[p] = dv[i];
    if (weighted) w[p] = wt[i];
  }
  std::vector<uint64_t> keep_oids = ctx->oids;
  sg_status st = load_csr(ctx, n, rp.data(), col.data(), weighted ? w.data() : nullptr);
  ctx->oids = keep_oids;  // load_csr resets the graph state
  return st;
}

sg_status read_update_file(sg_ctx* ctx, const char* path, std::vector<sg_update>* out) {
  FileBuf b = read_all(path);
  if (!b.ok) return fail(ctx, SG_ERR_INVALID, std::string("cannot read update file ") + path);
  Cursor c = cursor(b);
  while (!c.at_end()) {
    const char op = *c.p;
    if (op != 'a' && op != 'd')
      return fail(ctx, SG_ERR_INVALID, std::string("update lines start with 'a' or 'd': ") + path);
    ++c.p;
    uint64_t u, v;
    if (!c.read_u64(&u) || !c.read_u64(&v))
      return fail(ctx, SG_ERR_INVALID, std::string("malformed update line in ") + path);
    double w = 1.0;
    if (op == 'a' && c.line_has_more() && !c.read_f64(&w))
      return fail(ctx, SG_ERR_INVALID, std::string("malformed update weight in ") + path);
    sg_update r;
    if (!oid_to_vid(ctx, u, &r.src) || !oid_to_vid(ctx, v, &r.dst))
      return fail(ctx, SG_ERR_INVALID, "update names a vertex that is not in the graph");
    r.weight = (float)w;
    r.op = op == 'a' ? SG_UPD_ADD : SG_UPD_DEL;
    out->push_back(r);
    c.next_line();
  }
  return SG_OK;
}

sg_status read_cluster_file(sg_ctx* ctx, const char* path,
                            std::vector<std::vector<uint32_t>>* clusters) {
  FileBuf b = read_all(path);
  if (!b.ok) return fail(ctx, SG_ERR_INVALID, std::string("cannot read cluster file ") + path);
  Cursor c = cursor(b);
  while (!c.at_end()) {
    uint64_t size;
    if (!c.read_u64(&size)) return fail(ctx, SG_ERR_INVALID, "malformed cluster record");
    std::vector<uint32_t> members;
    members.reserve((size_t)size);
    for (uint64_t i = 0; i < size; ++i) {
      c.skip_blank();
      uint64_t o;
      uint32_t v;
      if (!c.read_u64(&o)) return fail(ctx, SG_ERR_INVALID, "cluster record shorter than its size");
      if (!oid_to_vid(ctx, o, &v))
        return fail(ctx, SG_ERR_INVALID, "cluster member that is not in the graph");
      members.push_back(v);
    }
    clusters->push_back(std::move(members));
  }
  return SG_OK;
}

}  // namespace sg
