// Object store behind the HDF5 stand-in (stand_in/hdf5.h).  Test infrastructure only.
//
// A file is a tree of groups whose leaves are datasets; datasets carry
// attributes.  The tree is loaded when a file is opened and saved when a file
// opened for writing is closed.  Handles are small integers into one table.
#include "hdf5.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

struct Blob {                 // typed array (dataset or attribute payload)
  hid_t type = 0;             // native id, or H5T_C_S1 for strings
  size_t esize = 0;           // element size in bytes
  std::vector<hsize_t> dims;  // empty = scalar
  std::vector<unsigned char> bytes;
  size_t count() const {
    size_t n = 1;
    for (hsize_t d : dims) n *= (size_t)d;
    return n;
  }
};

struct Node {
  bool is_group = true;
  std::map<std::string, std::unique_ptr<Node>> kids;  // groups
  Blob data;                                          // datasets
  std::map<std::string, Blob> attrs;                  // datasets
};

struct File {
  std::string path;
  bool writable = false;
  Node root;
};

enum Kind { K_FILE, K_GROUP, K_DSET, K_SPACE, K_ATTR, K_TYPE, K_PLIST };

struct Handle {
  explicit Handle(Kind k = K_PLIST) : kind(k) {}
  Kind kind;
  File* file = nullptr;   // K_FILE (owning through g_files)
  Node* node = nullptr;   // K_GROUP, K_DSET, K_ATTR (the dataset)
  std::string attr;       // K_ATTR
  std::vector<hsize_t> dims;  // K_SPACE
  bool scalar = false;        // K_SPACE
  hid_t type = 0;             // K_TYPE: base type
  size_t tsize = 0;           // K_TYPE: string size
};

std::map<hid_t, Handle> g_h;
std::map<hid_t, std::unique_ptr<File>> g_files;
hid_t g_next = 100000;

hid_t add(const Handle& h) {
  hid_t id = g_next++;
  g_h[id] = h;
  return id;
}
Handle* get(hid_t id) {
  auto it = g_h.find(id);
  return it == g_h.end() ? nullptr : &it->second;
}

size_t native_size(hid_t t) {
  switch (t) {
    case H5T_NATIVE_CHAR: case H5T_NATIVE_UCHAR: return 1;
    case H5T_NATIVE_SHORT: case H5T_NATIVE_USHORT: return sizeof(short);
    case H5T_NATIVE_INT: case H5T_NATIVE_UINT: return sizeof(int);
    case H5T_NATIVE_LONG: case H5T_NATIVE_ULONG: return sizeof(long);
    case H5T_NATIVE_LLONG: case H5T_NATIVE_ULLONG: return sizeof(long long);
    case H5T_NATIVE_FLOAT: return sizeof(float);
    case H5T_NATIVE_DOUBLE: return sizeof(double);
    case H5T_NATIVE_LDOUBLE: return sizeof(long double);
  }
  return 0;
}

// Resolve a type argument: a native id, or a string-type handle.
bool resolve_type(hid_t t, hid_t* base, size_t* esize) {
  if (size_t s = native_size(t)) { *base = t; *esize = s; return true; }
  if (t == H5T_C_S1) { *base = H5T_C_S1; *esize = 1; return true; }
  Handle* h = get(t);
  if (!h || h->kind != K_TYPE) return false;
  *base = h->type;
  *esize = h->tsize;
  return true;
}

bool is_float(hid_t t) { return t == H5T_NATIVE_FLOAT || t == H5T_NATIVE_DOUBLE || t == H5T_NATIVE_LDOUBLE; }

long double load_num(hid_t t, const unsigned char* p) {
  switch (t) {
    case H5T_NATIVE_CHAR: return *(const signed char*)p;
    case H5T_NATIVE_UCHAR: return *(const unsigned char*)p;
    case H5T_NATIVE_SHORT: return *(const short*)p;
    case H5T_NATIVE_USHORT: return *(const unsigned short*)p;
    case H5T_NATIVE_INT: return *(const int*)p;
    case H5T_NATIVE_UINT: return *(const unsigned*)p;
    case H5T_NATIVE_LONG: return *(const long*)p;
    case H5T_NATIVE_ULONG: return *(const unsigned long*)p;
    case H5T_NATIVE_LLONG: return *(const long long*)p;
    case H5T_NATIVE_ULLONG: return *(const unsigned long long*)p;
    case H5T_NATIVE_FLOAT: return *(const float*)p;
    case H5T_NATIVE_DOUBLE: return *(const double*)p;
    case H5T_NATIVE_LDOUBLE: return *(const long double*)p;
  }
  return 0;
}

void store_num(hid_t t, unsigned char* p, long double v) {
  switch (t) {
    case H5T_NATIVE_CHAR: *(signed char*)p = (signed char)v; break;
    case H5T_NATIVE_UCHAR: *(unsigned char*)p = (unsigned char)v; break;
    case H5T_NATIVE_SHORT: *(short*)p = (short)v; break;
    case H5T_NATIVE_USHORT: *(unsigned short*)p = (unsigned short)v; break;
    case H5T_NATIVE_INT: *(int*)p = (int)v; break;
    case H5T_NATIVE_UINT: *(unsigned*)p = (unsigned)v; break;
    case H5T_NATIVE_LONG: *(long*)p = (long)v; break;
    case H5T_NATIVE_ULONG: *(unsigned long*)p = (unsigned long)v; break;
    case H5T_NATIVE_LLONG: *(long long*)p = (long long)v; break;
    case H5T_NATIVE_ULLONG: *(unsigned long long*)p = (unsigned long long)v; break;
    case H5T_NATIVE_FLOAT: *(float*)p = (float)v; break;
    case H5T_NATIVE_DOUBLE: *(double*)p = (double)v; break;
    case H5T_NATIVE_LDOUBLE: *(long double*)p = v; break;
  }
}

// Copy n elements between typed buffers, converting numerics as HDF5 does.
bool convert(hid_t st, size_t ssz, const unsigned char* src, hid_t dt, size_t dsz, unsigned char* dst, size_t n) {
  if (st == dt && ssz == dsz) { std::memcpy(dst, src, n * ssz); return true; }
  if (st == H5T_C_S1 || dt == H5T_C_S1) {  // strings: copy, pad with zeros
    for (size_t i = 0; i < n; ++i) {
      std::memset(dst + i * dsz, 0, dsz);
      std::memcpy(dst + i * dsz, src + i * ssz, ssz < dsz ? ssz : dsz);
    }
    return true;
  }
  (void)is_float;
  for (size_t i = 0; i < n; ++i) store_num(dt, dst + i * dsz, load_num(st, src + i * ssz));
  return true;
}

// Walk a path ("/a/b/", "a", "/") from a file or group handle.
Node* walk(hid_t loc, const char* name, bool want_parent = false, std::string* leaf = nullptr) {
  Handle* h = get(loc);
  if (!h) return nullptr;
  Node* base = nullptr;
  std::string p = name ? name : "";
  if (h->kind == K_FILE) base = &h->file->root;
  else if (h->kind == K_GROUP) base = h->node;
  else return nullptr;
  if (!p.empty() && p[0] == '/') {
    File* f = h->file;
    base = &f->root;
  }
  std::vector<std::string> parts;
  size_t i = 0;
  while (i < p.size()) {
    size_t j = p.find('/', i);
    if (j == std::string::npos) j = p.size();
    if (j > i && p.substr(i, j - i) != ".") parts.push_back(p.substr(i, j - i));
    i = j + 1;
  }
  size_t stop = parts.size();
  if (want_parent) {
    if (parts.empty()) return nullptr;
    stop = parts.size() - 1;
    if (leaf) *leaf = parts.back();
  }
  Node* n = base;
  for (size_t k = 0; k < stop; ++k) {
    if (!n->is_group) return nullptr;
    auto it = n->kids.find(parts[k]);
    if (it == n->kids.end()) return nullptr;
    n = it->second.get();
  }
  return n;
}

File* file_of(hid_t loc) {
  Handle* h = get(loc);
  return h ? h->file : nullptr;
}

// ---- persistence (private layout) -------------------------------------------------------
void put_u64(FILE* f, uint64_t v) { std::fwrite(&v, 8, 1, f); }
bool get_u64(FILE* f, uint64_t* v) { return std::fread(v, 8, 1, f) == 1; }
void put_str(FILE* f, const std::string& s) { put_u64(f, s.size()); std::fwrite(s.data(), 1, s.size(), f); }
bool get_str(FILE* f, std::string* s) {
  uint64_t n;
  if (!get_u64(f, &n)) return false;
  s->assign(n, '\0');
  return n == 0 || std::fread(&(*s)[0], 1, n, f) == n;
}
void put_blob(FILE* f, const Blob& b) {
  put_u64(f, (uint64_t)b.type); put_u64(f, b.esize); put_u64(f, b.dims.size());
  for (hsize_t d : b.dims) put_u64(f, d);
  put_u64(f, b.bytes.size());
  if (!b.bytes.empty()) std::fwrite(b.bytes.data(), 1, b.bytes.size(), f);
}
bool get_blob(FILE* f, Blob* b) {
  uint64_t t, es, nd, nb;
  if (!get_u64(f, &t) || !get_u64(f, &es) || !get_u64(f, &nd)) return false;
  b->type = (hid_t)t; b->esize = es; b->dims.resize(nd);
  for (auto& d : b->dims) { uint64_t v; if (!get_u64(f, &v)) return false; d = v; }
  if (!get_u64(f, &nb)) return false;
  b->bytes.resize(nb);
  return nb == 0 || std::fread(b->bytes.data(), 1, nb, f) == nb;
}
void put_node(FILE* f, const Node& n) {
  put_u64(f, n.is_group ? 1 : 0);
  if (n.is_group) {
    put_u64(f, n.kids.size());
    for (auto& kv : n.kids) { put_str(f, kv.first); put_node(f, *kv.second); }
  } else {
    put_blob(f, n.data);
    put_u64(f, n.attrs.size());
    for (auto& kv : n.attrs) { put_str(f, kv.first); put_blob(f, kv.second); }
  }
}
bool get_node(FILE* f, Node* n) {
  uint64_t g;
  if (!get_u64(f, &g)) return false;
  n->is_group = g != 0;
  uint64_t cnt;
  if (n->is_group) {
    if (!get_u64(f, &cnt)) return false;
    for (uint64_t i = 0; i < cnt; ++i) {
      std::string name;
      if (!get_str(f, &name)) return false;
      std::unique_ptr<Node> k(new Node);
      if (!get_node(f, k.get())) return false;
      n->kids[name] = std::move(k);
    }
  } else {
    if (!get_blob(f, &n->data) || !get_u64(f, &cnt)) return false;
    for (uint64_t i = 0; i < cnt; ++i) {
      std::string name;
      Blob b;
      if (!get_str(f, &name) || !get_blob(f, &b)) return false;
      n->attrs[name] = std::move(b);
    }
  }
  return true;
}
const char kMagic[8] = {'P', 'C', 'F', 'D', 'H', '5', 'S', '1'};

}  // namespace

herr_t H5Eset_auto1(H5E_auto1_t, void*) { return 0; }

hid_t H5Fcreate(const char* name, unsigned flags, hid_t, hid_t) {
  if (flags & H5F_ACC_EXCL) {
    if (FILE* f = std::fopen(name, "rb")) { std::fclose(f); return -1; }
  }
  std::unique_ptr<File> fl(new File);
  fl->path = name;
  fl->writable = true;
  Handle h(K_FILE);
  h.file = fl.get();
  hid_t id = add(h);
  g_files[id] = std::move(fl);
  // Create the file on disk at once, as HDF5 does.
  if (FILE* f = std::fopen(name, "wb")) { std::fwrite(kMagic, 1, 8, f); put_node(f, g_files[id]->root); std::fclose(f); }
  else { g_h.erase(id); g_files.erase(id); return -1; }
  return id;
}

hid_t H5Fopen(const char* name, unsigned flags, hid_t) {
  FILE* f = std::fopen(name, "rb");
  if (!f) return -1;
  char magic[8];
  std::unique_ptr<File> fl(new File);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 && get_node(f, &fl->root);
  std::fclose(f);
  if (!ok) return -1;
  fl->path = name;
  fl->writable = (flags & H5F_ACC_RDWR) != 0;
  Handle h(K_FILE);
  h.file = fl.get();
  hid_t id = add(h);
  g_files[id] = std::move(fl);
  return id;
}

herr_t H5Fclose(hid_t id) {
  auto it = g_files.find(id);
  if (it == g_files.end()) return -1;
  File* fl = it->second.get();
  herr_t rc = 0;
  if (fl->writable) {
    FILE* f = std::fopen(fl->path.c_str(), "wb");
    if (!f) rc = -1;
    else { std::fwrite(kMagic, 1, 8, f); put_node(f, fl->root); std::fclose(f); }
  }
  // Handles into this file become invalid.
  for (auto h = g_h.begin(); h != g_h.end();) {
    if (h->second.file == fl && h->first != id) h = g_h.erase(h);
    else ++h;
  }
  g_h.erase(id);
  g_files.erase(it);
  return rc;
}

hid_t H5Gopen2(hid_t loc, const char* name, hid_t) {
  Node* n = walk(loc, name);
  if (!n || !n->is_group) return -1;
  Handle h(K_GROUP);
  h.file = file_of(loc);
  h.node = n;
  return add(h);
}

hid_t H5Gcreate2(hid_t loc, const char* name, hid_t, hid_t, hid_t) {
  std::string leaf;
  Node* parent = walk(loc, name, true, &leaf);
  if (!parent || !parent->is_group || parent->kids.count(leaf)) return -1;
  std::unique_ptr<Node> g(new Node);
  Node* raw = g.get();
  parent->kids[leaf] = std::move(g);
  Handle h(K_GROUP);
  h.file = file_of(loc);
  h.node = raw;
  return add(h);
}

herr_t H5Gclose(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_GROUP) return -1;
  g_h.erase(id);
  return 0;
}

herr_t H5Gget_objinfo(hid_t loc, const char* name, int, H5G_stat_t* st) {
  Node* n = walk(loc, name);
  if (!n) return -1;
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->type = n->is_group ? H5G_GROUP : H5G_DATASET;
    st->nlink = 1;
  }
  return 0;
}

herr_t H5Literate(hid_t group, H5_index_t, H5_iter_order_t, hsize_t* idx, H5L_iterate_t op, void* op_data) {
  Handle* h = get(group);
  if (!h) return -1;
  Node* n = h->kind == K_FILE ? &h->file->root : h->node;
  if (!n || !n->is_group) return -1;
  std::vector<std::string> names;
  for (auto& kv : n->kids) names.push_back(kv.first);  // map order = increasing name
  hsize_t k = 0;
  for (const std::string& nm : names) {
    H5L_info_t info;
    std::memset(&info, 0, sizeof(info));
    herr_t r = op(group, nm.c_str(), &info, op_data);
    ++k;
    if (r != 0) { if (idx) *idx = k; return r; }
  }
  if (idx) *idx = k;
  return 0;
}

hid_t H5Screate(H5S_class_t type) {
  Handle h(K_SPACE);
  h.scalar = (type == H5S_SCALAR);
  return add(h);
}

hid_t H5Screate_simple(int rank, const hsize_t* dims, const hsize_t*) {
  Handle h(K_SPACE);
  h.dims.assign(dims, dims + rank);
  return add(h);
}

herr_t H5Sclose(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_SPACE) return -1;
  g_h.erase(id);
  return 0;
}

int H5Sget_simple_extent_ndims(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_SPACE) return -1;
  return (int)h->dims.size();
}

int H5Sget_simple_extent_dims(hid_t id, hsize_t* dims, hsize_t* maxdims) {
  Handle* h = get(id);
  if (!h || h->kind != K_SPACE) return -1;
  for (size_t i = 0; i < h->dims.size(); ++i) {
    if (dims) dims[i] = h->dims[i];
    if (maxdims) maxdims[i] = h->dims[i];
  }
  return (int)h->dims.size();
}

herr_t H5Sselect_hyperslab(hid_t id, H5S_seloper_t, const hsize_t*, const hsize_t*, const hsize_t*, const hsize_t*) {
  return get(id) ? 0 : -1;  // whole-extent selections only
}

hid_t H5Tcopy(hid_t type) {
  hid_t base;
  size_t es;
  if (!resolve_type(type, &base, &es)) return -1;
  Handle h(K_TYPE);
  h.type = base;
  h.tsize = es;
  return add(h);
}

herr_t H5Tset_size(hid_t id, size_t size) {
  Handle* h = get(id);
  if (!h || h->kind != K_TYPE) return -1;
  h->tsize = size;
  return 0;
}

size_t H5Tget_size(hid_t id) {
  hid_t base;
  size_t es;
  return resolve_type(id, &base, &es) ? es : 0;
}

herr_t H5Tclose(hid_t id) {
  Handle* h = get(id);
  if (h && h->kind == K_TYPE) g_h.erase(id);
  return 0;
}

hid_t H5Pcreate(hid_t) { Handle h(K_PLIST); return add(h); }
herr_t H5Pset_buffer(hid_t, size_t, void*, void*) { return 0; }
herr_t H5Pclose(hid_t id) {
  Handle* h = get(id);
  if (h && h->kind == K_PLIST) g_h.erase(id);
  return 0;
}

hid_t H5Dopen2(hid_t loc, const char* name, hid_t) {
  Node* n = walk(loc, name);
  if (!n || n->is_group) return -1;
  Handle h(K_DSET);
  h.file = file_of(loc);
  h.node = n;
  return add(h);
}

hid_t H5Dcreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t, hid_t, hid_t) {
  std::string leaf;
  Node* parent = walk(loc, name, true, &leaf);
  Handle* sp = get(space);
  hid_t base;
  size_t es;
  if (!parent || !parent->is_group || parent->kids.count(leaf) || !sp || sp->kind != K_SPACE ||
      !resolve_type(type, &base, &es))
    return -1;
  std::unique_ptr<Node> d(new Node);
  d->is_group = false;
  d->data.type = base;
  d->data.esize = es;
  d->data.dims = sp->dims;
  d->data.bytes.assign(d->data.count() * es, 0);
  Node* raw = d.get();
  parent->kids[leaf] = std::move(d);
  Handle h(K_DSET);
  h.file = file_of(loc);
  h.node = raw;
  return add(h);
}

herr_t H5Dclose(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_DSET) return -1;
  g_h.erase(id);
  return 0;
}

hid_t H5Dget_type(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_DSET) return -1;
  if (native_size(h->node->data.type)) return h->node->data.type;
  Handle t(K_TYPE);
  t.type = h->node->data.type;
  t.tsize = h->node->data.esize;
  return add(t);
}

hid_t H5Dget_space(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_DSET) return -1;
  Handle s(K_SPACE);
  s.dims = h->node->data.dims;
  s.scalar = s.dims.empty();
  return add(s);
}

herr_t H5Dread(hid_t id, hid_t mem_type, hid_t, hid_t, hid_t, void* buf) {
  Handle* h = get(id);
  hid_t base;
  size_t es;
  if (!h || h->kind != K_DSET || !resolve_type(mem_type, &base, &es)) return -1;
  const Blob& b = h->node->data;
  convert(b.type, b.esize, b.bytes.data(), base, es, (unsigned char*)buf, b.count());
  return 0;
}

herr_t H5Dwrite(hid_t id, hid_t mem_type, hid_t, hid_t file_space, hid_t, const void* buf) {
  Handle* h = get(id);
  hid_t base;
  size_t es;
  if (!h || h->kind != K_DSET || !resolve_type(mem_type, &base, &es)) return -1;
  Blob& b = h->node->data;
  if (Handle* fs = get(file_space)) {  // an explicit file space may resize a re-opened dataset
    if (fs->kind == K_SPACE && !fs->scalar && fs->dims != b.dims) {
      b.dims = fs->dims;
      b.bytes.assign(b.count() * b.esize, 0);
    }
  }
  convert(base, es, (const unsigned char*)buf, b.type, b.esize, b.bytes.data(), b.count());
  return 0;
}

hid_t H5Acreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t, hid_t) {
  Handle* d = get(loc);
  Handle* sp = get(space);
  hid_t base;
  size_t es;
  if (!d || d->kind != K_DSET || !sp || sp->kind != K_SPACE || !resolve_type(type, &base, &es)) return -1;
  if (d->node->attrs.count(name)) return -1;
  Blob b;
  b.type = base;
  b.esize = es;
  b.dims = sp->dims;
  b.bytes.assign(b.count() * es, 0);
  d->node->attrs[name] = b;
  Handle a(K_ATTR);
  a.file = d->file;
  a.node = d->node;
  a.attr = name;
  return add(a);
}

hid_t H5Aopen(hid_t loc, const char* name, hid_t) {
  Handle* d = get(loc);
  if (!d || d->kind != K_DSET || !d->node->attrs.count(name)) return -1;
  Handle a(K_ATTR);
  a.file = d->file;
  a.node = d->node;
  a.attr = name;
  return add(a);
}

herr_t H5Adelete(hid_t loc, const char* name) {
  Handle* d = get(loc);
  if (!d || d->kind != K_DSET) return -1;
  return d->node->attrs.erase(name) ? 0 : -1;
}

herr_t H5Aclose(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_ATTR) return -1;
  g_h.erase(id);
  return 0;
}

hid_t H5Aget_type(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_ATTR) return -1;
  const Blob& b = h->node->attrs[h->attr];
  if (native_size(b.type)) return b.type;
  Handle t(K_TYPE);
  t.type = b.type;
  t.tsize = b.esize;
  return add(t);
}

hid_t H5Aget_space(hid_t id) {
  Handle* h = get(id);
  if (!h || h->kind != K_ATTR) return -1;
  Handle s(K_SPACE);
  s.dims = h->node->attrs[h->attr].dims;
  s.scalar = s.dims.empty();
  return add(s);
}

herr_t H5Aread(hid_t id, hid_t mem_type, void* buf) {
  Handle* h = get(id);
  hid_t base;
  size_t es;
  if (!h || h->kind != K_ATTR || !resolve_type(mem_type, &base, &es)) return -1;
  const Blob& b = h->node->attrs[h->attr];
  convert(b.type, b.esize, b.bytes.data(), base, es, (unsigned char*)buf, b.count());
  return 0;
}

herr_t H5Awrite(hid_t id, hid_t mem_type, const void* buf) {
  Handle* h = get(id);
  hid_t base;
  size_t es;
  if (!h || h->kind != K_ATTR || !resolve_type(mem_type, &base, &es)) return -1;
  Blob& b = h->node->attrs[h->attr];
  convert(base, es, (const unsigned char*)buf, b.type, b.esize, b.bytes.data(), b.count());
  return 0;
}
