// Tuning table: the launch shapes and limits of the kernels.
//
// The reference picks one shape by rule (setnb, hessenberg.jl:133-142: the
// panel width from n).  Here every shape that a measurement decides is a key of
// one table per handle: the defaults compiled in below are the values measured
// best on GB300; a table written by the autotuner (skewgpu/autotune.py, which
// times the library's own calls at each candidate value) replaces them for the
// device whose name it was measured on; skew_tuning_set changes one key.
//
// Table file (JSON): {"devices": {"<device name>": {"<key>": <int> | [<int>, ...],
// ...}, ...}, ...}; other members are ignored.  A handle loads, at creation, the
// file the environment variable SKEW_TUNING_FILE names, or else skew_tuning.json
// in the directory of libskewgpu.so, if the file holds an entry for the
// handle's device.  A key the file gives out of range makes the whole load fail
// (the handle keeps the defaults and reports the error through
// skew_tuning_source).
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <stdint.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/skewgpu.h"
#include "skew_internal.h"

namespace skew {

void tuning_defaults(Tuning* T) {
  *T = Tuning();
  const int edges[] = {32, 64, 96, 128, 152};
  T->nedges = 5;
  for (int i = 0; i < 5; i++) T->bucket_edges[i] = edges[i];
  T->batch_smem_nmax = 96;
  T->batch_smem_nt_small = 128;
  T->batch_smem_nt_large = 256;
  T->batch_global_nt = 256;
  T->batch_global_ctas_per_sm = 2;
  T->batch_graph = 1;
  T->batch_merge_global = 1;
  T->batch_split_pct = 50;
  T->func_chain_nmax = 64;
  T->func_real_schur = 1;
  T->blocked_min_n = 192;
  T->blocked_persistent = 1;
  T->cluster_max_n = 640;
  T->persist_ctas = 0;
  T->persist_tail = 0;
  T->persist_items = 8;
  T->persist_nb = 64;
  T->zpersist_min_n = 384;
  T->zpersist_ctas = 0;
  T->zpersist_items = 4;
  T->zpersist_nb = 32;
  T->pfz_cta_max = 160;
  T->pfz_nt = 0;
  T->pfz_ctas = 0;
  T->wait_polls = 0;
  T->wait_skip_cta = -1;
  T->qr_max_iter = 0;
}

namespace {

struct Key {
  const char* name;
  int Tuning::*field;  // null for the list and the 64-bit keys
  long long lo, hi;
  const int* allowed;  // null: any value in [lo, hi]
  int nallowed;
};

const int k128_256[] = {128, 256};
const int k256_512[] = {256, 512};
const int k01[] = {0, 1};
const int kpfz_nt[] = {0, 64, 128, 256, 512};

const Key kKeys[] = {
    {"bucket_edges", nullptr, 2, 1024, nullptr, 0},
    {"batch_smem_nmax", &Tuning::batch_smem_nmax, 0, 152, nullptr, 0},
    {"batch_smem_nt_small", &Tuning::batch_smem_nt_small, 128, 256, k128_256, 2},
    {"batch_smem_nt_large", &Tuning::batch_smem_nt_large, 256, 512, k256_512, 2},
    {"batch_global_nt", &Tuning::batch_global_nt, 256, 512, k256_512, 2},
    {"batch_global_ctas_per_sm", &Tuning::batch_global_ctas_per_sm, 1, 4, nullptr, 0},
    {"batch_graph", &Tuning::batch_graph, 0, 1, k01, 2},
    {"batch_merge_global", &Tuning::batch_merge_global, 0, 1, k01, 2},
    {"batch_split_pct", &Tuning::batch_split_pct, 0, 95, nullptr, 0},
    {"func_chain_nmax", &Tuning::func_chain_nmax, 0, 1 << 20, nullptr, 0},
    {"func_real_schur", &Tuning::func_real_schur, 0, 1, k01, 2},
    {"blocked_min_n", &Tuning::blocked_min_n, 16, 1025, nullptr, 0},
    {"blocked_persistent", &Tuning::blocked_persistent, 0, 1, k01, 2},
    {"cluster_max_n", &Tuning::cluster_max_n, 0, 640, nullptr, 0},
    {"persist_ctas", &Tuning::persist_ctas, 0, 1 << 16, nullptr, 0},
    {"persist_tail", &Tuning::persist_tail, 0, 1024, nullptr, 0},
    {"persist_items", &Tuning::persist_items, 1, 16, nullptr, 0},
    {"persist_nb", &Tuning::persist_nb, 8, 128, nullptr, 0},
    {"zpersist_min_n", &Tuning::zpersist_min_n, 129, 1 << 15, nullptr, 0},
    {"zpersist_ctas", &Tuning::zpersist_ctas, 0, 1 << 16, nullptr, 0},
    {"zpersist_items", &Tuning::zpersist_items, 1, 8, nullptr, 0},
    {"zpersist_nb", &Tuning::zpersist_nb, 4, 32, nullptr, 0},
    {"pfz_cta_max", &Tuning::pfz_cta_max, 0, 160, nullptr, 0},
    {"pfz_nt", &Tuning::pfz_nt, 0, 512, kpfz_nt, 5},
    {"pfz_ctas", &Tuning::pfz_ctas, 0, 1 << 16, nullptr, 0},
    {"wait_polls", nullptr, 0, 1LL << 40, nullptr, 0},
    {"wait_skip_cta", &Tuning::wait_skip_cta, -1, 1 << 20, nullptr, 0},
    {"qr_max_iter", &Tuning::qr_max_iter, 0, 1 << 30, nullptr, 0},
};

const Key* find_key(const char* name) {
  if (!name) return nullptr;
  for (const Key& k : kKeys)
    if (std::strcmp(k.name, name) == 0) return &k;
  return nullptr;
}

bool value_ok(const Key& k, long long v) {
  if (v < k.lo || v > k.hi) return false;
  if (!k.allowed) return true;
  for (int i = 0; i < k.nallowed; i++)
    if (k.allowed[i] == v) return true;
  return false;
}

}  // namespace

int tuning_set(Tuning* T, const char* key, const long long* v, int count) {
  const Key* k = find_key(key);
  if (!T || !k || !v || count < 1) return SKEW_BAD_ARG;
  if (std::strcmp(k->name, "bucket_edges") == 0) {
    if (count > kMaxBucketEdges) return SKEW_BAD_ARG;
    for (int i = 0; i < count; i++)
      if (!value_ok(*k, v[i]) || (i > 0 && v[i] <= v[i - 1])) return SKEW_BAD_ARG;
    T->nedges = count;
    for (int i = 0; i < count; i++) T->bucket_edges[i] = (int)v[i];
    return SKEW_OK;
  }
  if (count != 1 || !value_ok(*k, v[0])) return SKEW_BAD_ARG;
  if (k->field)
    T->*(k->field) = (int)v[0];
  else
    T->wait_polls = v[0];  // the one 64-bit key
  return SKEW_OK;
}

int tuning_get(const Tuning* T, const char* key, long long* v, int cap, int* count) {
  const Key* k = find_key(key);
  if (!T || !k || !v || cap < 1) return SKEW_BAD_ARG;
  if (std::strcmp(k->name, "bucket_edges") == 0) {
    if (count) *count = T->nedges;
    for (int i = 0; i < T->nedges && i < cap; i++) v[i] = T->bucket_edges[i];
    return SKEW_OK;
  }
  v[0] = k->field ? (long long)(T->*(k->field)) : T->wait_polls;
  if (count) *count = 1;
  return SKEW_OK;
}

const char* tuning_key_name(int i) {
  return (i >= 0 && i < (int)(sizeof(kKeys) / sizeof(kKeys[0]))) ? kKeys[i].name : nullptr;
}

// ---------------------------------------------------------------------------
// A small JSON reader: objects, arrays, strings, numbers, true/false/null.  It
// keeps only what the table needs: the members of devices[<name>] whose values
// are integers or arrays of integers.
// ---------------------------------------------------------------------------
namespace {

struct Reader {
  const char* p;
  const char* end;
  bool ok = true;

  void ws() {
    while (p < end && std::isspace((unsigned char)*p)) p++;
  }
  bool eat(char c) {
    ws();
    if (p < end && *p == c) {
      p++;
      return true;
    }
    return false;
  }
  bool string(std::string* out) {
    ws();
    if (p >= end || *p != '"') return ok = false;
    p++;
    std::string s;
    while (p < end && *p != '"') {
      if (*p == '\\' && p + 1 < end) {
        p++;
        const char e = *p;
        s.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
      } else {
        s.push_back(*p);
      }
      p++;
    }
    if (p >= end) return ok = false;
    p++;
    if (out) *out = s;
    return true;
  }
  bool number(double* out) {
    ws();
    char* q = nullptr;
    const double v = std::strtod(p, &q);
    if (q == p || q > end) return ok = false;
    p = q;
    if (out) *out = v;
    return true;
  }
  // skip any value
  bool skip() {
    ws();
    if (p >= end) return ok = false;
    if (*p == '"') return string(nullptr);
    if (*p == '{') {
      p++;
      if (eat('}')) return true;
      do {
        if (!string(nullptr) || !eat(':') || !skip()) return ok = false;
      } while (eat(','));
      return eat('}') || (ok = false);
    }
    if (*p == '[') {
      p++;
      if (eat(']')) return true;
      do {
        if (!skip()) return ok = false;
      } while (eat(','));
      return eat(']') || (ok = false);
    }
    for (const char* w : {"true", "false", "null"}) {
      const size_t l = std::strlen(w);
      if ((size_t)(end - p) >= l && std::strncmp(p, w, l) == 0) {
        p += l;
        return true;
      }
    }
    return number(nullptr);
  }
  // an integer or an array of integers
  bool ints(std::vector<long long>* out) {
    ws();
    out->clear();
    double d = 0.0;
    if (p < end && *p == '[') {
      p++;
      if (eat(']')) return true;
      do {
        if (!number(&d)) return false;
        out->push_back((long long)d);
        if ((double)out->back() != d) return ok = false;
      } while (eat(','));
      return eat(']') || (ok = false);
    }
    if (!number(&d)) return false;
    out->push_back((long long)d);
    return (double)out->back() == d || (ok = false);
  }
};

// Apply the members of the object at r.p (the device's entry) to T.
bool apply_entry(Reader& r, Tuning* T) {
  if (!r.eat('{')) return false;
  if (r.eat('}')) return true;
  do {
    std::string key;
    if (!r.string(&key) || !r.eat(':')) return false;
    if (find_key(key.c_str())) {
      std::vector<long long> v;
      if (!r.ints(&v) || v.empty()) return false;
      if (tuning_set(T, key.c_str(), v.data(), (int)v.size()) != SKEW_OK) return false;
    } else if (!r.skip()) {  // notes, measurements: not keys
      return false;
    }
  } while (r.eat(','));
  return r.eat('}');
}

}  // namespace

int tuning_load_file(Tuning* T, const char* path, const char* device, bool* found) {
  if (found) *found = false;
  if (!T || !path || !device) return SKEW_BAD_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return SKEW_BAD_ARG;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  Reader r{text.data(), text.data() + text.size()};
  Tuning next = *T;
  if (!r.eat('{')) return SKEW_BAD_ARG;
  if (r.eat('}')) return SKEW_OK;
  do {
    std::string top;
    if (!r.string(&top) || !r.eat(':')) return SKEW_BAD_ARG;
    if (top != "devices") {
      if (!r.skip()) return SKEW_BAD_ARG;
      continue;
    }
    if (!r.eat('{')) return SKEW_BAD_ARG;
    if (r.eat('}')) continue;
    do {
      std::string name;
      if (!r.string(&name) || !r.eat(':')) return SKEW_BAD_ARG;
      if (name == device) {
        if (!apply_entry(r, &next)) return SKEW_BAD_ARG;
        if (found) *found = true;
      } else if (!r.skip()) {
        return SKEW_BAD_ARG;
      }
    } while (r.eat(','));
    if (!r.eat('}')) return SKEW_BAD_ARG;
  } while (r.eat(','));
  if (!r.eat('}') || !r.ok) return SKEW_BAD_ARG;
  *T = next;
  return SKEW_OK;
}

// The table a new handle loads: SKEW_TUNING_FILE, else skew_tuning.json beside the library.
std::string tuning_default_path() {
  const char* env = std::getenv("SKEW_TUNING_FILE");
  if (env && *env) return env;
  Dl_info info;
  if (dladdr((const void*)&tuning_defaults, &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    const size_t slash = p.find_last_of('/');
    return (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/skew_tuning.json";
  }
  return "skew_tuning.json";
}

}  // namespace skew
