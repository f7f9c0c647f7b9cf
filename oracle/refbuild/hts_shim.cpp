// Clean-room implementation of the htslib API subset declared in include/htslib/*.h, so that breseq's
// own sources (error_count.cpp, identify_mutations.cpp, stats.cpp, pileup*.cpp, alignment.cpp, ...)
// compile and run unchanged as the reference oracle.  Test infrastructure only: nothing in the
// product links it.  It follows the SAM/BAM format specification (SAMv1: BGZF blocks, the binary
// record layout, auxiliary fields) and the behaviour htslib documents for the calls breseq makes:
//   - hts_open / sam_hdr_read / sam_read1: the whole BGZF file is inflated with zlib on open and the
//     records are read in file order;
//   - sam_index_load / sam_itr_queryi / sam_itr_next: no .bai is read; an iterator scans the file for
//     records of the target whose alignment overlaps [beg, end) (an alignment with no reference-
//     consuming operation covers one base);
//   - bam_plp_*: htslib's pileup, the default filter mask UNMAP | SECONDARY | QCFAIL | DUP, one column
//     per reference position that some kept record covers, in increasing position, each column listing
//     the covering records in the order they were read, with
//       qpos   the query index of the base (M / = / X), or for a deletion / skip column the query
//              index the operation starts at (the next aligned base),
//       indel  at the last column of an operation: minus the summed lengths of the D operations that
//              follow, or the summed lengths of the I operations that follow (P operations skipped);
//              0 otherwise,
//       is_del / is_refskip  the column lies in a D / N operation, is_head / is_tail  the first / last
//              column of the alignment;
//   - fai_*: the FASTA file is parsed whole; sequences are returned as NUL-terminated copies.
#include <zlib.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "htslib/faidx.h"
#include "htslib/sam.h"

namespace {

bool read_file(const char* fn, std::vector<uint8_t>& out) {
  FILE* f = fopen(fn, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  size_t got = n > 0 ? fread(out.data(), 1, (size_t)n, f) : 0;
  fclose(f);
  return got == out.size();
}

// BGZF: a series of gzip members, each with a BC extra subfield holding its size minus one.
bool inflate_bgzf(const std::vector<uint8_t>& in, std::vector<uint8_t>& out) {
  size_t pos = 0;
  out.clear();
  while (pos + 18 <= in.size()) {
    const uint8_t* h = in.data() + pos;
    if (h[0] != 31 || h[1] != 139 || h[2] != 8 || !(h[3] & 4)) return false;
    const uint32_t xlen = h[10] | (h[11] << 8);
    uint32_t bsize = 0;
    for (uint32_t x = 0; x + 4 <= xlen;) {
      const uint8_t* sf = h + 12 + x;
      const uint32_t slen = sf[2] | (sf[3] << 8);
      if (sf[0] == 'B' && sf[1] == 'C' && slen == 2) bsize = (sf[4] | (sf[5] << 8)) + 1u;
      x += 4 + slen;
    }
    if (bsize == 0 || pos + bsize > in.size()) return false;
    const uint32_t isize = h[bsize - 4] | (h[bsize - 3] << 8) | (h[bsize - 2] << 16) | ((uint32_t)h[bsize - 1] << 24);
    const size_t cdata = 12 + xlen, clen = bsize - cdata - 8;
    const size_t o = out.size();
    out.resize(o + isize);
    if (isize) {
      z_stream z;
      memset(&z, 0, sizeof z);
      if (inflateInit2(&z, -15) != Z_OK) return false;
      z.next_in = const_cast<Bytef*>(h + cdata);
      z.avail_in = (uInt)clen;
      z.next_out = out.data() + o;
      z.avail_out = isize;
      const int r = inflate(&z, Z_FINISH);
      inflateEnd(&z);
      if (r != Z_STREAM_END || z.avail_out != 0) return false;
    }
    pos += bsize;
  }
  return pos == in.size();
}

template <class T> T rd(const uint8_t* p) { T v; memcpy(&v, p, sizeof v); return v; }

// Parses the SAM header text into its lines and tags (the @RG lookups breseq makes).
struct HeaderLines {
  struct Line { std::string type; std::vector<std::pair<std::string, std::string>> tags; };
  std::vector<Line> lines;
  void parse(const char* text, size_t n) {
    lines.clear();
    size_t i = 0;
    while (i < n && text[i]) {
      size_t j = i;
      while (j < n && text[j] && text[j] != '\n') j++;
      std::string l(text + i, j - i);
      if (l.size() > 3 && l[0] == '@') {
        Line L;
        L.type = l.substr(1, 2);
        size_t k = 3;
        while (k < l.size()) {
          if (l[k] == '\t') { k++; continue; }
          size_t e = l.find('\t', k);
          if (e == std::string::npos) e = l.size();
          const std::string f = l.substr(k, e - k);
          if (f.size() >= 3 && f[2] == ':') L.tags.emplace_back(f.substr(0, 2), f.substr(3));
          k = e;
        }
        lines.push_back(L);
      }
      i = j + 1;
    }
  }
  const Line* nth(const char* type, int pos) const {
    int c = 0;
    for (const Line& L : lines)
      if (L.type == type && c++ == pos) return &L;
    return nullptr;
  }
};

}  // namespace

struct hts_file_s {
  std::vector<uint8_t> data;   // the inflated BGZF stream
  size_t off = 0;              // next record
  size_t first = 0;            // first record (after the header)
  std::string fn;
};
struct hts_idx_s { std::string fn; };
struct hts_itr_s {
  std::vector<uint8_t> data;
  size_t off = 0;
  int tid = 0;
  hts_pos_t beg = 0, end = 0;
};

extern "C" {

// ------------------------------------------------------------------------------- files, headers
htsFile* hts_open(const char* fn, const char* mode) {
  if (!fn || !mode || mode[0] != 'r') return nullptr;   // reading only
  std::vector<uint8_t> raw;
  if (!read_file(fn, raw)) return nullptr;
  htsFile* f = new hts_file_s();
  f->fn = fn;
  if (!inflate_bgzf(raw, f->data) || f->data.size() < 4 || memcmp(f->data.data(), "BAM\1", 4) != 0) {
    delete f;
    return nullptr;
  }
  return f;
}

int hts_close(htsFile* fp) { delete fp; return 0; }
int hts_set_opt(htsFile*, enum hts_fmt_option, ...) { return 0; }

static sam_hdr_t* new_header(const char* text, size_t l_text) {
  sam_hdr_t* h = (sam_hdr_t*)calloc(1, sizeof(sam_hdr_t));
  h->l_text = l_text;
  h->text = (char*)malloc(l_text + 1);
  memcpy(h->text, text, l_text);
  h->text[l_text] = 0;
  HeaderLines* hl = new HeaderLines();
  hl->parse(h->text, l_text);
  h->hrecs = hl;
  return h;
}

sam_hdr_t* sam_hdr_init(void) { return new_header("", 0); }

sam_hdr_t* sam_hdr_read(samFile* fp) {
  if (!fp) return nullptr;
  const uint8_t* d = fp->data.data();
  const size_t n = fp->data.size();
  size_t p = 4;
  if (p + 4 > n) return nullptr;
  const int32_t l_text = rd<int32_t>(d + p);
  p += 4;
  if (l_text < 0 || p + (size_t)l_text + 4 > n) return nullptr;
  sam_hdr_t* h = new_header((const char*)d + p, strnlen((const char*)d + p, (size_t)l_text));
  p += (size_t)l_text;
  const int32_t n_ref = rd<int32_t>(d + p);
  p += 4;
  h->n_targets = n_ref;
  h->target_len = (uint32_t*)calloc((size_t)n_ref + 1, sizeof(uint32_t));
  h->target_name = (char**)calloc((size_t)n_ref + 1, sizeof(char*));
  for (int32_t i = 0; i < n_ref; i++) {
    const int32_t l_name = rd<int32_t>(d + p);
    p += 4;
    h->target_name[i] = strndup((const char*)d + p, (size_t)l_name);
    p += (size_t)l_name;
    h->target_len[i] = rd<uint32_t>(d + p);
    p += 4;
  }
  fp->off = fp->first = p;
  return h;
}

// @SQ lines give the targets of a text header (SN name, LN length)
sam_hdr_t* sam_hdr_parse(size_t l_text, const char* text) {
  sam_hdr_t* h = new_header(text, l_text);
  const HeaderLines* hl = (const HeaderLines*)h->hrecs;
  std::vector<std::pair<std::string, uint32_t>> sq;
  for (const auto& L : hl->lines) {
    if (L.type != "SQ") continue;
    std::string sn;
    uint32_t ln = 0;
    for (const auto& t : L.tags) {
      if (t.first == "SN") sn = t.second;
      if (t.first == "LN") ln = (uint32_t)strtoul(t.second.c_str(), nullptr, 10);
    }
    sq.emplace_back(sn, ln);
  }
  h->n_targets = (int32_t)sq.size();
  h->target_len = (uint32_t*)calloc(sq.size() + 1, sizeof(uint32_t));
  h->target_name = (char**)calloc(sq.size() + 1, sizeof(char*));
  for (size_t i = 0; i < sq.size(); i++) { h->target_name[i] = strdup(sq[i].first.c_str()); h->target_len[i] = sq[i].second; }
  return h;
}

void sam_hdr_destroy(sam_hdr_t* h) {
  if (!h) return;
  for (int32_t i = 0; i < h->n_targets; i++) free(h->target_name[i]);
  free(h->target_name);
  free(h->target_len);
  free(h->text);
  delete (HeaderLines*)h->hrecs;
  free(h);
}

int sam_hdr_count_lines(sam_hdr_t* h, const char* type) {
  if (!h || !type) return -1;
  int c = 0;
  for (const auto& L : ((const HeaderLines*)h->hrecs)->lines) c += L.type == type;
  return c;
}

// the identifying tag of the pos-th line of a type: ID for @RG (SN for @SQ)
const char* sam_hdr_line_name(sam_hdr_t* h, const char* type, int pos) {
  if (!h || !type) return nullptr;
  const HeaderLines::Line* L = ((const HeaderLines*)h->hrecs)->nth(type, pos);
  if (!L) return nullptr;
  const char* key = strcmp(type, "SQ") == 0 ? "SN" : "ID";
  for (const auto& t : L->tags)
    if (t.first == key) return t.second.c_str();
  return nullptr;
}

int sam_hdr_find_tag_pos(sam_hdr_t* h, const char* type, int pos, const char* key, kstring_t* ks) {
  if (!h || !type || !key || !ks) return -2;
  const HeaderLines::Line* L = ((const HeaderLines*)h->hrecs)->nth(type, pos);
  if (!L) return -1;
  for (const auto& t : L->tags)
    if (t.first == key) {
      ks->l = 0;
      kputs(t.second.c_str(), ks);
      return 0;
    }
  return -1;
}

int sam_hdr_write(samFile*, const sam_hdr_t*) { return -1; }      // writing is not on the oracle's path
int sam_write1(samFile*, const sam_hdr_t*, const bam1_t*) { return -1; }
int sam_parse1(kstring_t*, sam_hdr_t*, bam1_t*) { return -1; }
int bam_sort_core(int, const char*, const char*, size_t) { return -1; }

// ------------------------------------------------------------------------------- records
bam1_t* bam_init1(void) { return (bam1_t*)calloc(1, sizeof(bam1_t)); }

void bam_destroy1(bam1_t* b) {
  if (!b) return;
  free(b->data);
  free(b);
}

bam1_t* bam_copy1(bam1_t* dst, const bam1_t* src) {
  uint8_t* d = dst->data;
  uint32_t m = dst->m_data;
  if (m < (uint32_t)src->l_data) {
    m = (uint32_t)src->l_data + 32;
    d = (uint8_t*)realloc(d, m);
  }
  memcpy(d, src->data, (size_t)src->l_data);
  *dst = *src;
  dst->data = d;
  dst->m_data = m;
  return dst;
}

hts_pos_t bam_cigar2qlen(int n, const uint32_t* c) {
  hts_pos_t l = 0;
  for (int k = 0; k < n; k++)
    if (bam_cigar_type(bam_cigar_op(c[k])) & 1) l += bam_cigar_oplen(c[k]);
  return l;
}

hts_pos_t bam_cigar2rlen(int n, const uint32_t* c) {
  hts_pos_t l = 0;
  for (int k = 0; k < n; k++)
    if (bam_cigar_type(bam_cigar_op(c[k])) & 2) l += bam_cigar_oplen(c[k]);
  return l;
}

hts_pos_t bam_endpos(const bam1_t* b) {
  hts_pos_t rl = 0;
  if (!(b->core.flag & BAM_FUNMAP)) rl = bam_cigar2rlen((int)b->core.n_cigar, bam_get_cigar(b));
  if (rl == 0) rl = 1;
  return b->core.pos + rl;
}

// decodes the record at data[off]; returns its size (>0) or -1 at the end of the data
static int decode_record(const std::vector<uint8_t>& data, size_t& off, bam1_t* b) {
  if (off + 4 > data.size()) return -1;
  const uint8_t* p = data.data() + off;
  const int32_t bs = rd<int32_t>(p);
  if (bs < 32 || off + 4 + (size_t)bs > data.size()) return -1;
  bam1_core_t& c = b->core;
  c.tid = rd<int32_t>(p + 4);
  c.pos = rd<int32_t>(p + 8);
  c.l_qname = p[12];
  c.qual = p[13];
  c.bin = rd<uint16_t>(p + 14);
  c.n_cigar = rd<uint16_t>(p + 16);
  c.flag = rd<uint16_t>(p + 18);
  c.l_qseq = rd<int32_t>(p + 20);
  c.mtid = rd<int32_t>(p + 24);
  c.mpos = rd<int32_t>(p + 28);
  c.isize = rd<int32_t>(p + 32);
  c.l_extranul = 0;
  const int l = bs - 32;
  if ((uint32_t)l + 1 > b->m_data) {
    b->m_data = (uint32_t)l + 64;
    b->data = (uint8_t*)realloc(b->data, b->m_data);
  }
  memcpy(b->data, p + 36, (size_t)l);
  b->l_data = l;
  off += 4 + (size_t)bs;
  return bs + 4;
}

int sam_read1(samFile* fp, sam_hdr_t*, bam1_t* b) {
  if (!fp || !b) return -2;
  return decode_record(fp->data, fp->off, b);
}

// ------------------------------------------------------------------------------- aux fields
static size_t aux_size(const uint8_t* s, const uint8_t* end) {   // s at the type byte
  switch (*s) {
    case 'A': case 'c': case 'C': return 2;
    case 's': case 'S': return 3;
    case 'i': case 'I': case 'f': return 5;
    case 'd': return 9;
    case 'Z': case 'H': {
      const uint8_t* q = s + 1;
      while (q < end && *q) q++;
      return (size_t)(q - s) + 1;
    }
    case 'B': {
      const uint8_t sub = s[1];
      const uint32_t n = rd<uint32_t>(s + 2);
      const size_t w = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2 : 4;
      return 6 + w * n;
    }
    default: return (size_t)(end - s);
  }
}

uint8_t* bam_aux_get(const bam1_t* b, const char tag[2]) {
  uint8_t* s = bam_get_aux(b);
  uint8_t* end = b->data + b->l_data;
  while (s + 3 <= end) {
    if (s[0] == tag[0] && s[1] == tag[1]) return s + 2;
    s += 2 + aux_size(s + 2, end);
  }
  return nullptr;
}

int64_t bam_aux2i(const uint8_t* s) {
  if (!s) return 0;
  switch (*s) {
    case 'c': return (int8_t)s[1];
    case 'C': return s[1];
    case 's': return rd<int16_t>(s + 1);
    case 'S': return rd<uint16_t>(s + 1);
    case 'i': return rd<int32_t>(s + 1);
    case 'I': return rd<uint32_t>(s + 1);
    default: return 0;
  }
}

char* bam_aux2Z(const uint8_t* s) {
  if (!s || (*s != 'Z' && *s != 'H')) return nullptr;
  return (char*)s + 1;
}

int bam_aux_del(bam1_t* b, uint8_t* s) {   // s at the type byte of the field to remove
  uint8_t* start = s - 2;
  uint8_t* end = b->data + b->l_data;
  const size_t n = 2 + aux_size(s, end);
  memmove(start, start + n, (size_t)(end - start - n));
  b->l_data -= (int)n;
  return 0;
}

int bam_aux_append(bam1_t* b, const char tag[2], char type, int len, const uint8_t* data) {
  const uint32_t need = (uint32_t)b->l_data + 3 + (uint32_t)len;
  if (need > b->m_data) {
    b->m_data = need + 32;
    b->data = (uint8_t*)realloc(b->data, b->m_data);
  }
  uint8_t* p = b->data + b->l_data;
  p[0] = (uint8_t)tag[0]; p[1] = (uint8_t)tag[1]; p[2] = (uint8_t)type;
  memcpy(p + 3, data, (size_t)len);
  b->l_data = (int)need;
  return 0;
}

// ------------------------------------------------------------------------------- index, iterators
hts_idx_t* sam_index_load(htsFile* fp, const char* fn) {
  if (!fp || !fn) return nullptr;
  hts_idx_t* i = new hts_idx_s();
  i->fn = fn;
  return i;
}

void hts_idx_destroy(hts_idx_t* idx) { delete idx; }

hts_itr_t* sam_itr_queryi(const hts_idx_t* idx, int tid, hts_pos_t beg, hts_pos_t end) {
  if (!idx) return nullptr;
  htsFile* f = hts_open(idx->fn.c_str(), "rb");
  if (!f) return nullptr;
  sam_hdr_t* h = sam_hdr_read(f);
  if (!h) { hts_close(f); return nullptr; }
  hts_itr_t* it = new hts_itr_s();
  it->data.swap(f->data);
  it->off = f->first;
  it->tid = tid; it->beg = beg; it->end = end;
  sam_hdr_destroy(h);
  hts_close(f);
  return it;
}

int sam_itr_next(htsFile*, hts_itr_t* it, bam1_t* b) {
  if (!it) return -2;
  for (;;) {
    const int r = decode_record(it->data, it->off, b);
    if (r < 0) return -1;
    if (b->core.tid < it->tid || b->core.tid < 0) continue;
    if (b->core.tid > it->tid || b->core.pos >= it->end) return -1;   // coordinate-sorted: past the region
    if (bam_endpos(b) > it->beg) return r;
  }
}

void hts_itr_destroy(hts_itr_t* it) { delete it; }

// ------------------------------------------------------------------------------- pileup
struct bam_plp_s {
  bam_plp_auto_f func;
  void* data;
  uint32_t mask = BAM_FUNMAP | BAM_FSECONDARY | BAM_FQCFAIL | BAM_FDUP;
  struct Act {
    bam1_t* b;
    hts_pos_t end;   // exclusive end column
  };
  std::deque<Act> act;               // records covering or ahead of the column, in read order
  bam1_t* next = nullptr;            // read but not yet entered
  bool eof = false;
  int tid = -1;
  hts_pos_t pos = 0;
  std::vector<bam_pileup1_t> out;
};

bam_plp_t bam_plp_init(bam_plp_auto_f func, void* data) {
  bam_plp_t it = new bam_plp_s();
  it->func = func;
  it->data = data;
  return it;
}

void bam_plp_set_maxcnt(bam_plp_t, int) {}

void bam_plp_destroy(bam_plp_t it) {
  if (!it) return;
  for (auto& a : it->act) bam_destroy1(a.b);
  if (it->next) bam_destroy1(it->next);
  delete it;
}

static void plp_fetch(bam_plp_t it) {   // the next kept record into it->next, or eof
  if (it->next || it->eof) return;
  bam1_t* b = bam_init1();
  for (;;) {
    if (it->func(it->data, b) < 0) { bam_destroy1(b); it->eof = true; return; }
    if (b->core.tid < 0 || (b->core.flag & it->mask)) continue;
    it->next = b;
    return;
  }
}

// the pileup entry of record b at column pos (pos inside [b.pos, endpos))
static bool plp_resolve(const bam1_t* b, hts_pos_t pos, hts_pos_t endpos, bam_pileup1_t& p) {
  const uint32_t* cg = bam_get_cigar(b);
  const int n = (int)b->core.n_cigar;
  hts_pos_t x = b->core.pos;
  int32_t y = 0;
  memset(&p, 0, sizeof p);
  p.b = const_cast<bam1_t*>(b);
  for (int k = 0; k < n; k++) {
    const uint32_t op = bam_cigar_op(cg[k]), l = bam_cigar_oplen(cg[k]);
    const int t = bam_cigar_type(op);
    if (t & 2) {                       // consumes the reference
      if (pos < x + (hts_pos_t)l) {
        if (t & 1) p.qpos = y + (int32_t)(pos - x);
        else { p.qpos = y; p.is_del = 1; p.is_refskip = op == BAM_CREF_SKIP; }
        p.cigar_ind = k;
        if (pos == x + (hts_pos_t)l - 1 && k + 1 < n) {
          const uint32_t op2 = bam_cigar_op(cg[k + 1]);
          if (op2 == BAM_CDEL && op != BAM_CDEL) {
            int d = 0;
            for (int j = k + 1; j < n && bam_cigar_op(cg[j]) == BAM_CDEL; j++) d += (int)bam_cigar_oplen(cg[j]);
            p.indel = -d;
          } else if (op2 == BAM_CINS || op2 == BAM_CPAD) {
            int ins = 0;
            for (int j = k + 1; j < n; j++) {
              const uint32_t o = bam_cigar_op(cg[j]);
              if (o == BAM_CINS) ins += (int)bam_cigar_oplen(cg[j]);
              else if (o != BAM_CPAD) break;
            }
            p.indel = ins;
          }
        }
        p.is_head = pos == b->core.pos;
        p.is_tail = pos == endpos - 1;
        return true;
      }
      x += l;
    }
    if (t & 1) y += (int32_t)l;
  }
  return false;
}

const bam_pileup1_t* bam_plp_auto(bam_plp_t it, int* tid, int* pos, int* n_plp) {
  for (;;) {
    plp_fetch(it);
    // drop records that end at or before the column
    std::deque<bam_plp_s::Act> keep;
    for (auto& a : it->act) {
      if (a.end > it->pos) keep.push_back(a);
      else bam_destroy1(a.b);
    }
    it->act.swap(keep);
    if (it->act.empty()) {
      if (!it->next) { *n_plp = 0; return nullptr; }
      it->tid = it->next->core.tid;
      it->pos = it->next->core.pos;
    }
    // enter the records that start at or before the column on this target
    while (it->next && it->next->core.tid == it->tid && it->next->core.pos <= it->pos) {
      it->act.push_back({it->next, bam_endpos(it->next)});
      it->next = nullptr;
      plp_fetch(it);
    }
    it->out.clear();
    for (auto& a : it->act) {
      if (a.b->core.pos > it->pos || a.end <= it->pos) continue;
      bam_pileup1_t p;
      if (plp_resolve(a.b, it->pos, a.end, p)) it->out.push_back(p);
    }
    const int c_tid = it->tid;
    const hts_pos_t c_pos = it->pos;
    it->pos++;
    if (!it->out.empty()) {
      *tid = c_tid;
      *pos = (int)c_pos;
      *n_plp = (int)it->out.size();
      return it->out.data();
    }
  }
}

}  // extern "C"

// ------------------------------------------------------------------------------- FASTA
struct faidx_s {
  std::vector<std::string> names;
  std::map<std::string, std::string> seq;
};

extern "C" {

faidx_t* fai_load(const char* fn) {
  FILE* f = fopen(fn, "r");
  if (!f) return nullptr;
  faidx_t* fai = new faidx_s();
  std::string name, cur;
  char buf[1 << 16];
  auto flush = [&]() { if (!name.empty()) { fai->names.push_back(name); fai->seq[name] = cur; } };
  while (fgets(buf, sizeof buf, f)) {
    size_t l = strlen(buf);
    while (l && (buf[l - 1] == '\n' || buf[l - 1] == '\r')) buf[--l] = 0;
    if (buf[0] == '>') {
      flush();
      name.assign(buf + 1);
      const size_t sp = name.find_first_of(" \t");
      if (sp != std::string::npos) name.resize(sp);
      cur.clear();
    } else {
      cur.append(buf, l);
    }
  }
  flush();
  fclose(f);
  return fai;
}

void fai_destroy(faidx_t* fai) { delete fai; }

char* faidx_fetch_seq(const faidx_t* fai, const char* name, int beg, int end, int* len) {
  auto i = fai->seq.find(name);
  if (i == fai->seq.end()) { if (len) *len = -2; return nullptr; }
  const std::string& s = i->second;
  if (beg < 0) beg = 0;
  if (end >= (int)s.size()) end = (int)s.size() - 1;
  const int n = end >= beg ? end - beg + 1 : 0;
  char* out = (char*)malloc((size_t)n + 1);
  memcpy(out, s.data() + beg, (size_t)n);
  out[n] = 0;
  if (len) *len = n;
  return out;
}

char* fai_fetch(const faidx_t* fai, const char* reg, int* len) {
  std::string r(reg);
  if (fai->seq.count(r)) return faidx_fetch_seq(fai, reg, 0, 0x7fffffff, len);
  const size_t colon = r.rfind(':');
  if (colon == std::string::npos) { if (len) *len = -2; return nullptr; }
  const std::string nm = r.substr(0, colon);
  int b = 1, e = 0x7fffffff;
  sscanf(r.c_str() + colon + 1, "%d-%d", &b, &e);
  return faidx_fetch_seq(fai, nm.c_str(), b - 1, e - 1, len);
}

int faidx_nseq(const faidx_t* fai) { return (int)fai->names.size(); }
const char* faidx_iseq(const faidx_t* fai, int i) { return fai->names[(size_t)i].c_str(); }
int faidx_seq_len(const faidx_t* fai, const char* seq) {
  auto i = fai->seq.find(seq);
  return i == fai->seq.end() ? -1 : (int)i->second.size();
}
int faidx_has_seq(const faidx_t* fai, const char* seq) { return fai->seq.count(seq) ? 1 : 0; }

}  // extern "C"
