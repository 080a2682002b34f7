// io.cu -- the data formats either side of the crmsd path, host C++.
//
// Multi-model ingestion.  The coordinates of every model of a PDB or mmCIF
// file, as bioshell-pdb keeps them (Structure::model_coordinates,
// structure.rs:100) without going through set_model per model:
//   * PDB (load_pdb.rs:52-115): ATOM/HETATM records; the atoms of the first
//     model define the atom list, ENDMDL starts the next model, coordinates
//     from columns 31-38, 39-46, 47-54 (Vec3::from_pdb_line, vec3.rs:241-246);
//   * mmCIF (pdb_atom.rs:130-170): the _atom_site loop; models in order of
//     first appearance of pdbx_PDB_model_num; atom names formatted from
//     label_atom_id and type_symbol (format_atom_name, pdb_atom.rs:306-331).
//   Selection "CA" keeps the atoms whose 4-character name is " CA "
//   (IsCA::check, pdb_atom_filters.rs:388-413), decided on the first model;
//   every model must hold the same atoms.  Decimal coordinates are converted
//   exactly (the correctly rounded double of the decimal string).
//
// Distance-matrix TSV, the input of the clust tool (clust.rs:102-105,
// tests/test_files/d5.tsv): one "label<TAB>label<TAB>value" line per pair.
//   * bs_tsv_write streams a packed triangle (host or device memory) in
//     chunks: device -> pinned host copies overlap the formatting, which runs
//     on all host threads; values are printed with a fixed number of
//     decimals, rounded to nearest (ties to even) from the exact binary value,
//     as printf("%.*f") prints them.
//   * bs_tsv_read: labels numbered in order of first appearance (row label,
//     then column label); the value of pair {i, j} is that of the line
//     (i, j) if present, else of (j, i) when the file is read as symmetric,
//     else the default value.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/bioshell_crmsd.h"

namespace {

thread_local std::string g_err;

bs_status io_err(bs_status s, const std::string &msg) {
  g_err = msg;
  return s;
}

bool read_file(const char *path, std::string &buf) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  if (fseek(f, 0, SEEK_END) != 0) {
    fclose(f);
    return false;
  }
  const long sz = ftell(f);
  if (sz < 0 || fseek(f, 0, SEEK_SET) != 0) {
    fclose(f);
    return false;
  }
  buf.resize((size_t)sz);
  const size_t got = sz > 0 ? fread(&buf[0], 1, (size_t)sz, f) : 0;
  fclose(f);
  return got == (size_t)sz;
}

// The correctly rounded double of a decimal token [p, e) ("-12.345",
// "1.5e-3", ...).  Plain decimals of up to 15 significant digits are
// converted exactly as m / 10^k (both exact doubles, one rounding); anything
// else goes through strtod.
bool parse_decimal(const char *p, const char *e, double &out) {
  while (p < e && (*p == ' ' || *p == '\t')) ++p;
  while (e > p && (e[-1] == ' ' || e[-1] == '\t' || e[-1] == '\r')) --e;
  if (p == e) return false;
  const char *q = p;
  bool neg = false;
  if (*q == '-' || *q == '+') neg = *q++ == '-';
  uint64_t m = 0;
  int digits = 0, frac = -1;
  bool simple = true;
  for (; q < e; ++q) {
    const char c = *q;
    if (c >= '0' && c <= '9') {
      if (m == 0 && c == '0' && frac < 0) continue;  // leading zeros
      m = m * 10 + (uint64_t)(c - '0');
      if (m != 0) ++digits;
      if (frac >= 0) ++frac;
    } else if (c == '.' && frac < 0) {
      frac = 0;
    } else {
      simple = false;
      break;
    }
  }
  static const double p10[] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11, 1e12, 1e13, 1e14, 1e15};
  if (simple && digits <= 15 && frac <= 15) {
    // fractional zeros after the leading ones still count in frac
    const double v = (double)m / p10[frac < 0 ? 0 : frac];
    out = neg ? -v : v;
    return true;
  }
  std::string s(p, e);
  char *end = nullptr;
  out = strtod(s.c_str(), &end);
  return end && *end == '\0';
}

// ------------------------------------------------------------------ models
struct Models {
  int64_t n = 0;
  int32_t L = 0;
  std::vector<double> xyz;  // [n][L][3]
};

bool is_cif_text(const std::string &b) {
  size_t i = 0;
  while (i < b.size()) {
    size_t j = b.find('\n', i);
    if (j == std::string::npos) j = b.size();
    size_t k = i;
    while (k < j && (b[k] == ' ' || b[k] == '\t' || b[k] == '\r')) ++k;
    if (k < j) return b.compare(i, 5, "data_") == 0;  // the first non-empty line
    i = j + 1;
  }
  return false;
}

bs_status read_pdb(const std::string &b, int selection, Models &out) {
  std::vector<char> keep;       // atoms of model 0 kept by the selection
  std::vector<std::vector<double>> models(1);
  size_t model = 0, atom_in_model = 0;
  size_t i = 0;
  int64_t line_no = 0;
  while (i < b.size()) {
    size_t j = b.find('\n', i);
    if (j == std::string::npos) j = b.size();
    const char *l = b.data() + i;
    size_t len = j - i;
    if (len > 0 && l[len - 1] == '\r') --len;
    ++line_no;
    if (len >= 6) {
      // the record name: the first six columns, trimmed
      int rl = 6;
      while (rl > 0 && l[rl - 1] == ' ') --rl;
      if ((rl == 4 && !strncmp(l, "ATOM", 4)) || (rl == 6 && !strncmp(l, "HETATM", 6))) {
        if (len < 54) return io_err(BS_ERR_INVALID_ARG, "line " + std::to_string(line_no) + ": ATOM record too short");
        double x, y, z;
        if (!parse_decimal(l + 30, l + 38, x) || !parse_decimal(l + 38, l + 46, y) || !parse_decimal(l + 46, l + 54, z))
          return io_err(BS_ERR_INVALID_ARG, "line " + std::to_string(line_no) + ": bad coordinates");
        bool k;
        if (model == 0) {
          k = selection == 0 || !strncmp(l + 12, " CA ", 4);
          keep.push_back(k ? 1 : 0);
        } else {
          if (atom_in_model >= keep.size())
            return io_err(BS_ERR_INVALID_ARG, "model " + std::to_string(model + 1) + " has more atoms than model 1");
          k = keep[atom_in_model] != 0;
        }
        ++atom_in_model;
        if (k) {
          models[model].push_back(x);
          models[model].push_back(y);
          models[model].push_back(z);
        }
      } else if (rl == 6 && !strncmp(l, "ENDMDL", 6)) {
        if (model > 0 && atom_in_model != keep.size())
          return io_err(BS_ERR_INVALID_ARG, "model " + std::to_string(model + 1) + " has fewer atoms than model 1");
        ++model;
        atom_in_model = 0;
        models.emplace_back();
      }
    }
    i = j + 1;
  }
  if (!models.empty() && models.back().empty() && atom_in_model == 0 && models.size() > 1) models.pop_back();
  if (models.size() > 1 && atom_in_model != 0 && atom_in_model != keep.size())
    return io_err(BS_ERR_INVALID_ARG, "last model has a different number of atoms");
  const size_t per = models[0].size();
  if (per == 0) return io_err(BS_ERR_INVALID_ARG, "no atoms selected");
  for (const auto &m : models)
    if (m.size() != per) return io_err(BS_ERR_INVALID_ARG, "models hold different numbers of atoms");
  out.n = (int64_t)models.size();
  out.L = (int32_t)(per / 3);
  out.xyz.reserve(per * models.size());
  for (const auto &m : models) out.xyz.insert(out.xyz.end(), m.begin(), m.end());
  return BS_OK;
}

// CIF tokens of one line: whitespace-separated, 'quoted' or "quoted" (a
// quote ends a token only when followed by whitespace or the line's end).
void cif_tokens(const char *l, size_t len, std::vector<std::pair<const char *, const char *>> &t) {
  size_t i = 0;
  while (i < len) {
    while (i < len && (l[i] == ' ' || l[i] == '\t' || l[i] == '\r')) ++i;
    if (i >= len) break;
    if (l[i] == '\'' || l[i] == '"') {
      const char q = l[i];
      size_t k = i + 1;
      while (k < len && !(l[k] == q && (k + 1 == len || l[k + 1] == ' ' || l[k + 1] == '\t' || l[k + 1] == '\r'))) ++k;
      t.emplace_back(l + i + 1, l + std::min(k, len));
      i = k + 1;
    } else {
      size_t k = i;
      while (k < len && l[k] != ' ' && l[k] != '\t' && l[k] != '\r') ++k;
      t.emplace_back(l + i, l + k);
      i = k;
    }
  }
}

// format_atom_name (pdb_atom.rs:306-331): the 4-character PDB atom name
void format_atom_name(const char *n, const char *ne, const char *el, const char *ele, char out[4]) {
  memset(out, ' ', 4);
  while (n < ne && *n == ' ') ++n;
  while (el < ele && *el == ' ') ++el;
  while (ele > el && ele[-1] == ' ') --ele;
  if (n >= ne) return;
  if (*n >= '0' && *n <= '9') {
    for (int i = 0; i < 4 && n + i < ne; ++i) out[i] = n[i];
    return;
  }
  const size_t elen = (size_t)(ele - el);
  const int pad = (elen == 0 || elen == 1) ? 1 : 0;
  for (int i = 0; i < 4 - pad && n + i < ne; ++i) out[pad + i] = n[i];
}

bs_status read_cif(const std::string &b, int selection, Models &out) {
  std::vector<std::string> cols;
  std::vector<std::pair<const char *, const char *>> tok, row;
  size_t i = 0;
  bool in_header = false, in_rows = false, done = false;
  int cx = -1, cy = -1, cz = -1, cname = -1, celem = -1, cmodel = -1;
  std::vector<long long> model_ids;                  // in order of first appearance
  std::unordered_map<long long, size_t> model_index;
  std::vector<std::vector<double>> models;
  std::vector<char> keep;                            // atoms of the first model kept
  std::vector<size_t> count;                         // atoms seen per model
  int64_t line_no = 0;
  auto flush_row = [&]() -> bs_status {
    const auto &t = row;
    long long mid = 1;
    if (cmodel >= 0) {
      double v;
      if (!parse_decimal(t[cmodel].first, t[cmodel].second, v)) return io_err(BS_ERR_INVALID_ARG, "bad model number");
      mid = (long long)v;
    }
    auto it = model_index.find(mid);
    size_t mi;
    if (it == model_index.end()) {
      mi = models.size();
      model_index.emplace(mid, mi);
      model_ids.push_back(mid);
      models.emplace_back();
      count.push_back(0);
    } else {
      mi = it->second;
    }
    double x, y, z;
    if (!parse_decimal(t[cx].first, t[cx].second, x) || !parse_decimal(t[cy].first, t[cy].second, y) ||
        !parse_decimal(t[cz].first, t[cz].second, z))
      return io_err(BS_ERR_INVALID_ARG, "line " + std::to_string(line_no) + ": bad coordinates");
    bool k;
    if (mi == 0) {
      char nm[4];
      const char *e0 = celem >= 0 ? t[celem].first : "", *e1 = celem >= 0 ? t[celem].second : e0;
      format_atom_name(t[cname].first, t[cname].second, e0, e1, nm);
      k = selection == 0 || !memcmp(nm, " CA ", 4);
      keep.push_back(k ? 1 : 0);
    } else {
      if (count[mi] >= keep.size()) return io_err(BS_ERR_INVALID_ARG, "a model has more atoms than the first");
      k = keep[count[mi]] != 0;
    }
    ++count[mi];
    if (k) {
      models[mi].push_back(x);
      models[mi].push_back(y);
      models[mi].push_back(z);
    }
    return BS_OK;
  };
  while (i < b.size() && !done) {
    size_t j = b.find('\n', i);
    if (j == std::string::npos) j = b.size();
    const char *l = b.data() + i;
    const size_t len = j - i;
    ++line_no;
    if (!in_header && !in_rows) {
      if (len >= 5 && !strncmp(l, "loop_", 5)) {
        // the next line tells whether this loop is _atom_site
        size_t k = j + 1;
        if (k < b.size() && b.compare(k, 11, "_atom_site.") == 0) in_header = true;
      }
    } else if (in_header) {
      if (len >= 11 && !strncmp(l, "_atom_site.", 11)) {
        size_t e = 11;
        while (e < len && l[e] != ' ' && l[e] != '\t' && l[e] != '\r') ++e;
        cols.emplace_back(l + 11, l + e);
      } else {
        in_header = false;
        in_rows = true;
        for (size_t c = 0; c < cols.size(); ++c) {
          if (cols[c] == "Cartn_x") cx = (int)c;
          else if (cols[c] == "Cartn_y") cy = (int)c;
          else if (cols[c] == "Cartn_z") cz = (int)c;
          else if (cols[c] == "label_atom_id") cname = (int)c;
          else if (cols[c] == "type_symbol") celem = (int)c;
          else if (cols[c] == "pdbx_PDB_model_num") cmodel = (int)c;
        }
        if (cx < 0 || cy < 0 || cz < 0 || cname < 0) return io_err(BS_ERR_INVALID_ARG, "_atom_site lacks coordinates or atom names");
        continue;  // re-read this line as a data row
      }
    } else {  // rows
      if (len == 0 || l[0] == '#' || (len >= 5 && !strncmp(l, "loop_", 5)) || l[0] == '_' ||
          (len >= 5 && !strncmp(l, "data_", 5))) {
        done = true;
        break;
      }
      tok.clear();
      cif_tokens(l, len, tok);
      for (const auto &t : tok) {
        row.push_back(t);
        if (row.size() == cols.size()) {
          const bs_status s = flush_row();
          if (s) return s;
          row.clear();
        }
      }
    }
    i = j + 1;
  }
  if (!row.empty()) return io_err(BS_ERR_INVALID_ARG, "truncated _atom_site row");
  if (models.empty() || models[0].empty()) return io_err(BS_ERR_INVALID_ARG, "no atoms selected");
  const size_t per = models[0].size();
  for (size_t m = 0; m < models.size(); ++m)
    if (models[m].size() != per || count[m] != keep.size())
      return io_err(BS_ERR_INVALID_ARG, "models hold different numbers of atoms");
  out.n = (int64_t)models.size();
  out.L = (int32_t)(per / 3);
  out.xyz.reserve(per * models.size());
  for (const auto &m : models) out.xyz.insert(out.xyz.end(), m.begin(), m.end());
  return BS_OK;
}

// ------------------------------------------------------------------ TSV
// v * 10^d rounded to nearest, ties to even, from the exact binary value.
// Returns false when |v| * 10^d does not fit 63 bits (caller falls back).
bool fixed_digits(double v, int d, bool &neg, unsigned long long &q) {
  if (!std::isfinite(v)) return false;
  neg = std::signbit(v);
  const double a = std::fabs(v);
  if (a == 0.0) {
    q = 0;
    return true;
  }
  int e;
  const double fr = std::frexp(a, &e);                     // a = fr 2^e, fr in [0.5, 1)
  const unsigned long long m = (unsigned long long)std::ldexp(fr, 53);  // a = m 2^(e-53)
  unsigned __int128 p5 = 1;
  for (int i = 0; i < d; ++i) p5 *= 5;                     // 10^d = 5^d 2^d
  const unsigned __int128 num = (unsigned __int128)m * p5; // a 10^d = num 2^(e-53+d)
  const int sh = e - 53 + d;
  if (sh >= 0) {
    if (sh > 60 || (num >> (63 - sh)) != 0) return false;
    q = (unsigned long long)(num << sh);
    return true;
  }
  const int r = -sh;
  if (r >= 127) {
    q = 0;
    return true;
  }
  const unsigned __int128 whole = num >> r;
  const unsigned __int128 rem = num - (whole << r);
  const unsigned __int128 half = (unsigned __int128)1 << (r - 1);
  unsigned __int128 w = whole;
  if (rem > half || (rem == half && (whole & 1))) w += 1;
  if ((w >> 63) != 0) return false;
  q = (unsigned long long)w;
  return true;
}

size_t format_value(double v, int d, char *out) {
  bool neg;
  unsigned long long q;
  if (!fixed_digits(v, d, neg, q)) return (size_t)snprintf(out, 64, "%.*f", d, v);
  char tmp[32];
  int k = 0;
  do {
    tmp[k++] = (char)('0' + q % 10);
    q /= 10;
  } while (q > 0 || k <= d);
  size_t o = 0;
  if (neg) out[o++] = '-';
  for (int i = k - 1; i >= d; --i) out[o++] = tmp[i];
  if (d > 0) {
    out[o++] = '.';
    for (int i = d - 1; i >= 0; --i) out[o++] = tmp[i];
  }
  return o;
}

struct Tsv {
  std::vector<std::string> labels;
  std::vector<float> tri;
};

bool is_device(const void *p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

struct bs_models {
  Models m;
};
struct bs_tsv {
  Tsv t;
};

extern "C" {

BS_API const char *bs_io_last_error(void) { return g_err.c_str(); }

BS_API bs_status bs_models_read(const char *path, int32_t format, int32_t selection, bs_models **out, int64_t *n_models,
                                int32_t *n_atoms) {
  if (!path || !out || !n_models || !n_atoms || format < 0 || format > 2 || selection < 0 || selection > 1)
    return io_err(BS_ERR_INVALID_ARG, "bad argument");
  *out = nullptr;
  std::string buf;
  if (!read_file(path, buf)) return io_err(BS_ERR_INVALID_ARG, std::string("cannot read ") + path);
  const bool cif = format == 2 || (format == 0 && is_cif_text(buf));
  bs_models *m = new (std::nothrow) bs_models;
  if (!m) return io_err(BS_ERR_OOM, "out of memory");
  bs_status s;
  try {
    s = cif ? read_cif(buf, selection, m->m) : read_pdb(buf, selection, m->m);
  } catch (const std::bad_alloc &) {
    s = io_err(BS_ERR_OOM, "out of memory");
  }
  if (s) {
    delete m;
    return s;
  }
  *out = m;
  *n_models = m->m.n;
  *n_atoms = m->m.L;
  return BS_OK;
}

BS_API bs_status bs_models_copy(const bs_models *m, double *xyz) {
  if (!m || !xyz) return io_err(BS_ERR_INVALID_ARG, "bad argument");
  if (cudaMemcpy(xyz, m->m.xyz.data(), m->m.xyz.size() * sizeof(double), cudaMemcpyDefault) != cudaSuccess) {
    cudaGetLastError();
    // host memory without a CUDA runtime: plain copy
    memcpy(xyz, m->m.xyz.data(), m->m.xyz.size() * sizeof(double));
  }
  return BS_OK;
}

BS_API void bs_models_free(bs_models *m) { delete m; }

BS_API bs_status bs_tsv_write(const char *path, const void *tri, int64_t n, int32_t out_type, const char *const *labels,
                              int32_t decimals) {
  if (!path || n < 0 || (n > 1 && !tri) || (out_type != BS_OUT_F64 && out_type != BS_OUT_F32))
    return io_err(BS_ERR_INVALID_ARG, "bad argument");
  const int d = decimals > 0 ? std::min(decimals, 17) : 6;
  FILE *f = fopen(path, "wb");
  if (!f) return io_err(BS_ERR_INVALID_ARG, std::string("cannot write ") + path);
  std::vector<std::string> lab((size_t)n);
  for (int64_t i = 0; i < n; ++i) lab[i] = labels && labels[i] ? std::string(labels[i]) : std::to_string(i);
  const size_t esz = out_type == BS_OUT_F64 ? 8 : 4;
  const int64_t total = n * (n - 1) / 2;
  const bool dev = n > 1 && is_device(tri);
  // rows are formatted in chunks of ~8M pairs; device chunks are staged in
  // two pinned buffers so that the next copy overlaps the formatting
  const int64_t chunk_pairs = (int64_t)8 << 20;
  const unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  void *stage[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bs_status status = BS_OK;
  if (dev) {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaHostAlloc(&stage[0], (size_t)chunk_pairs * esz, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&stage[1], (size_t)chunk_pairs * esz, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreate(&ev[0]) != cudaSuccess || cudaEventCreate(&ev[1]) != cudaSuccess) {
      cudaGetLastError();
      status = io_err(BS_ERR_CUDA, "staging buffers");
    }
  }
  // chunk boundaries at row starts
  std::vector<int64_t> row_start;  // first row of each chunk
  {
    int64_t r = 0, acc = 0;
    row_start.push_back(0);
    for (; r < n; ++r) {
      acc += n - 1 - r;
      if (acc >= chunk_pairs && r + 1 < n) {
        row_start.push_back(r + 1);
        acc = 0;
      }
    }
    row_start.push_back(n);
  }
  auto tri_off = [&](int64_t i) { return i * n - i * (i + 1) / 2; };
  auto enqueue = [&](size_t c, int slot) {
    const int64_t a = tri_off(row_start[c]), b = tri_off(row_start[c + 1]);
    cudaMemcpyAsync(stage[slot], static_cast<const char *>(tri) + a * esz, (size_t)(b - a) * esz,
                    cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ev[slot], st);
  };
  std::vector<std::string> parts(nth);
  if (status == BS_OK && dev && row_start.size() > 1 && row_start[0] < row_start[1]) enqueue(0, 0);
  for (size_t c = 0; status == BS_OK && c + 1 < row_start.size(); ++c) {
    const int64_t r0 = row_start[c], r1 = row_start[c + 1];
    const char *src;       // the chunk's values; entry idx of the triangle at src[idx - base]
    int64_t base = 0;
    if (dev) {
      const int slot = (int)(c & 1);
      if (cudaEventSynchronize(ev[slot]) != cudaSuccess) {
        status = io_err(BS_ERR_CUDA, "device copy");
        break;
      }
      if (c + 2 < row_start.size()) enqueue(c + 1, slot ^ 1);
      src = static_cast<const char *>(stage[slot]);
      base = tri_off(r0);
    } else {
      src = static_cast<const char *>(tri);
    }
    // rows of the chunk split over the threads by pair count
    std::vector<int64_t> cut(nth + 1, r1);
    cut[0] = r0;
    {
      const int64_t pairs = tri_off(r1) - tri_off(r0);
      int64_t acc = 0;
      unsigned t = 1;
      for (int64_t r = r0; r < r1 && t < nth; ++r) {
        acc += n - 1 - r;
        if (acc * (int64_t)nth >= pairs * (int64_t)t) cut[t++] = r + 1;
      }
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        std::string &o = parts[t];
        o.clear();
        char val[64];
        for (int64_t r = cut[t]; r < cut[t + 1]; ++r)
          for (int64_t c2 = r + 1; c2 < n; ++c2) {
            const int64_t idx = tri_off(r) + (c2 - r - 1) - base;
            const double v = esz == 8 ? reinterpret_cast<const double *>(src)[idx]
                                      : (double)reinterpret_cast<const float *>(src)[idx];
            o += lab[r];
            o += '\t';
            o += lab[c2];
            o += '\t';
            o.append(val, format_value(v, d, val));
            o += '\n';
          }
      });
    for (auto &x : th) x.join();
    for (const auto &o : parts)
      if (!o.empty() && fwrite(o.data(), 1, o.size(), f) != o.size()) {
        status = io_err(BS_ERR_INVALID_ARG, "write failed");
        break;
      }
  }
  if (fclose(f) != 0 && status == BS_OK) status = io_err(BS_ERR_INVALID_ARG, "write failed");
  if (dev) {
    if (st) cudaStreamSynchronize(st);
    for (void *p : stage)
      if (p) cudaFreeHost(p);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
  }
  return status;
}

BS_API bs_status bs_tsv_read(const char *path, double default_value, int32_t symmetric, bs_tsv **out, int64_t *n) {
  if (!path || !out || !n) return io_err(BS_ERR_INVALID_ARG, "bad argument");
  *out = nullptr;
  std::string buf;
  if (!read_file(path, buf)) return io_err(BS_ERR_INVALID_ARG, std::string("cannot read ") + path);
  bs_tsv *t = new (std::nothrow) bs_tsv;
  if (!t) return io_err(BS_ERR_OOM, "out of memory");
  try {
    std::unordered_map<std::string, int64_t> id;
    struct E {
      int64_t a, b;
      double v;
    };
    std::vector<E> es;
    size_t i = 0;
    int64_t line_no = 0;
    auto intern = [&](const char *p, const char *e) {
      std::string s(p, e);
      auto it = id.find(s);
      if (it != id.end()) return it->second;
      const int64_t k = (int64_t)t->t.labels.size();
      id.emplace(s, k);
      t->t.labels.push_back(std::move(s));
      return k;
    };
    while (i < buf.size()) {
      size_t j = buf.find('\n', i);
      if (j == std::string::npos) j = buf.size();
      ++line_no;
      const char *l = buf.data() + i;
      size_t len = j - i;
      while (len > 0 && (l[len - 1] == '\r' || l[len - 1] == ' ')) --len;
      if (len > 0 && l[0] != '#') {
        const char *p = l, *e = l + len;
        const char *t1 = (const char *)memchr(p, '\t', (size_t)(e - p));
        const char *t2 = t1 ? (const char *)memchr(t1 + 1, '\t', (size_t)(e - t1 - 1)) : nullptr;
        if (!t1 || !t2) {
          delete t;
          return io_err(BS_ERR_INVALID_ARG, "line " + std::to_string(line_no) + ": expected label<TAB>label<TAB>value");
        }
        const char *t3 = (const char *)memchr(t2 + 1, '\t', (size_t)(e - t2 - 1));
        double v;
        if (!parse_decimal(t2 + 1, t3 ? t3 : e, v)) {
          delete t;
          return io_err(BS_ERR_INVALID_ARG, "line " + std::to_string(line_no) + ": bad value");
        }
        const int64_t a = intern(p, t1), b = intern(t1 + 1, t2);
        es.push_back(E{a, b, v});
      }
      i = j + 1;
    }
    const int64_t m = (int64_t)t->t.labels.size();
    const int64_t tot = m * (m - 1) / 2;
    t->t.tri.assign((size_t)tot, (float)default_value);
    std::vector<char> direct((size_t)tot, 0);  // set by a line (i, j) with i < j
    for (const E &x : es) {
      if (x.a == x.b) continue;
      const int64_t lo = std::min(x.a, x.b), hi = std::max(x.a, x.b);
      const int64_t k = lo * m - lo * (lo + 1) / 2 + (hi - lo - 1);
      if (x.a < x.b) {
        t->t.tri[k] = (float)x.v;
        direct[k] = 1;
      } else if (symmetric && !direct[k]) {
        t->t.tri[k] = (float)x.v;
      }
    }
    *n = m;
  } catch (const std::bad_alloc &) {
    delete t;
    return io_err(BS_ERR_OOM, "out of memory");
  }
  *out = t;
  return BS_OK;
}

BS_API bs_status bs_tsv_matrix(const bs_tsv *t, float *tri) {
  if (!t || (!tri && !t->t.tri.empty())) return io_err(BS_ERR_INVALID_ARG, "bad argument");
  if (!t->t.tri.empty()) memcpy(tri, t->t.tri.data(), t->t.tri.size() * sizeof(float));
  return BS_OK;
}

BS_API const char *bs_tsv_label(const bs_tsv *t, int64_t i) {
  if (!t || i < 0 || i >= (int64_t)t->t.labels.size()) return nullptr;
  return t->t.labels[(size_t)i].c_str();
}

BS_API void bs_tsv_free(bs_tsv *t) { delete t; }

}  // extern "C"
