// Pipeline binding, planning and execution.
//
// bind()          mirrors Pipeline::Pipeline (core/pipeline.cu:11-80): operator
//                 dispatch and expression binding out of the PipelineInfo.
// run_select()    Source/Filter/Map/Sink pipelines (the dimension-side
//                 pipelines, e.g. example/run_SSB_Q31.cu:11-74): one
//                 order-preserving filter+project pass on the device.
// run_star()      Source/Filter/JoinWith/ReduceBy/Sink pipelines: dimension
//                 tables built (and cached) the way Pipeline::Open does
//                 (core/pipeline.cu:82-137) but on the device, then the fused
//                 scan of kern_star.cu replacing the generated loop and
//                 ReduceTask (core/pipeline.cu:262-472).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <set>
#include <unordered_map>

#include "ctx.h"
#include "expr.h"
#include "kernels.h"
#include "strdict.h"

namespace svm {

namespace {

struct Bound {
  std::string id;
  std::vector<std::string> select_exp, filter_exp, metric_exp;
  std::vector<ColRef> reduce_key, join_lkey, join_rkey;
  bool is_reduce = false;
  bool has_map = false;
  std::vector<svm_column_desc> sink;
  // Per ReduceBy key: for a String key (grouped by hash rank), the Hash value
  // of each rank, written in place of the rank; empty otherwise.
  std::vector<std::vector<int32_t>> key_hash;
};

const char* arg_of(const svm_operator& op, const char* key) {
  for (int k = 0; k < op.nargs; k++)
    if (op.args[k].key && std::strcmp(op.args[k].key, key) == 0) return op.args[k].value ? op.args[k].value : "";
  return nullptr;
}

svm_status bind(Ctx* x, const svm_pipeline* p, Bound* b) {
  b->id = p->id ? p->id : "";
  if (b->id.empty()) return x->fail(SVM_E_INVALID_ARG, "pipeline id is empty");
  bool has_sink = false;
  for (int i = 0; i < p->nops; i++) {
    const svm_operator& op = p->ops[i];
    std::string err;
    switch (op.type) {
      case SVM_OP_SOURCE:
        break;
      case SVM_OP_LOADER:
        return x->fail(SVM_E_UNSUPPORTED, "Loader (text parsing) pipelines are not part of this data plane; "
                                          "put columns with svm_object_put");
      case SVM_OP_SINK:
        has_sink = true;
        b->sink.assign(op.output, op.output + op.ncols);
        break;
      case SVM_OP_MAP: {
        const char* s = arg_of(op, "select");
        if (!s) return x->fail(SVM_E_INVALID_ARG, "Map without 'select'");
        b->select_exp = str_split(s, ",");
        b->has_map = true;
        break;
      }
      case SVM_OP_FILTER: {
        const char* s = arg_of(op, "predication");
        if (!s) return x->fail(SVM_E_INVALID_ARG, "Filter without 'predication'");
        b->filter_exp.push_back(s);
        break;
      }
      case SVM_OP_REDUCEBY: {
        const char* m = arg_of(op, "metric");
        if (!m) return x->fail(SVM_E_INVALID_ARG, "ReduceBy without 'metric'");
        b->metric_exp = str_split(m, ",");
        const char* d = arg_of(op, "dim");
        if (d) {
          for (auto& e : str_split(d, ",")) {
            ColRef r;
            if (!parse_key_index(e, &r, &err)) return x->fail(SVM_E_INVALID_ARG, "ReduceBy dim: " + err);
            b->reduce_key.push_back(r);
          }
        }
        b->is_reduce = true;
        break;
      }
      case SVM_OP_JOINWITH: {
        const char* l = arg_of(op, "lkey");
        const char* r = arg_of(op, "rkey");
        if (!l || !r) return x->fail(SVM_E_INVALID_ARG, "JoinWith needs 'lkey' and 'rkey'");
        ColRef lr, rr;
        if (!parse_key_index(l, &lr, &err) || !parse_key_index(r, &rr, &err))
          return x->fail(SVM_E_INVALID_ARG, "JoinWith: " + err);
        b->join_lkey.push_back(lr);
        b->join_rkey.push_back(rr);
        break;
      }
      case SVM_OP_SORTBY:
        break;  // ignored by the reference as well (core/pipeline.cu:69-71)
      default:
        return x->fail(SVM_E_INVALID_ARG, "unknown operator type " + std::to_string(op.type));
    }
  }
  if (!has_sink) return x->fail(SVM_E_INVALID_ARG, "pipeline has no Sink");
  return SVM_OK;
}

std::string join_filters(const std::vector<std::string>& f) {
  // Filters are concatenated with "&&", no parentheses (codegen/codegen.cpp:100-110).
  std::string s;
  for (size_t i = 0; i < f.size(); i++) {
    if (i) s += "&&";
    s += f[i];
  }
  return s;
}

int ceil_log2(unsigned long long v) {  // bits to hold values 0..v-1
  int b = 0;
  while (b < 64 && (1ull << b) < v) b++;
  return b;
}

svm_status sync_and_check(Ctx* x, const char* what) {
  cudaError_t e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, what);
  int h = 0;
  e = cudaMemcpy(&h, x->d_error, sizeof(int), cudaMemcpyDeviceToHost);
  if (e) return x->cuda_fail(e, what);
  if (h) {
    cudaMemset(x->d_error, 0, sizeof(int));
    const char* m;
    const svm_status s = device_error_status(h, &m);
    return x->fail(s, std::string(what) + ": " + m);
  }
  return SVM_OK;
}

ObjectPtr new_result_object(Ctx* x, const std::string& id, const std::vector<int>& types,
                            unsigned long long nrows, svm_status* st) {
  auto o = std::make_shared<Object>();
  o->id = id;
  o->version = x->next_version++;
  o->ncols = (int)types.size();
  o->types = types;
  o->nrows = nrows;
  o->source_rows = nrows;
  unsigned long long padded = (nrows + 63) / 64 * 64 + 64;
  for (int t : types) {
    DevBufPtr b;
    *st = x->alloc(padded * (t == SVM_INT64 ? 8 : 4), &b, true);
    if (*st) return nullptr;
    o->storage.push_back(b);
  }
  *st = SVM_OK;
  return o;
}

// ============================================================ select pipelines
svm_status build_dim(Ctx* x, const ObjectPtr& obj, int key_col, const std::vector<int>& pay_cols,
                     DimTablePtr* out);

// A Map pipeline, with or without joins.  With JoinWith operators the
// reference's generated loop probes each joined table after the conjuncts,
// drops a row whose key is missing, and projects expressions that may read
// the matched rows of the joined objects (codegen/codegen.cpp:121-180, the
// select block after the join block; rows written at j, j += cond).  Here
// the joined objects' tables carry the columns the projections read as
// payload, and the two-pass order-preserving compaction probes them per row.
svm_status run_select(Ctx* x, const Bound& b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs) {
  if (!b.has_map) return x->fail(SVM_E_UNSUPPORTED, "a pipeline without ReduceBy needs a Map");
  std::string err;
  std::vector<Expr> proj(b.select_exp.size());
  std::vector<ColRef> refs_used;
  for (size_t i = 0; i < b.select_exp.size(); i++) {
    if (!parse_expr(b.select_exp[i], &proj[i], &err))
      return x->fail(err.rfind("unsupported", 0) == 0 ? SVM_E_UNSUPPORTED : SVM_E_INVALID_ARG,
                     "select '" + b.select_exp[i] + "': " + err);
    collect_refs(proj[i], proj[i].root, &refs_used);
  }
  Expr pred;
  bool has_pred = !b.filter_exp.empty();
  std::vector<ColRef> pred_refs;
  if (has_pred) {
    std::string t = join_filters(b.filter_exp);
    if (!parse_expr(t, &pred, &err))
      return x->fail(err.rfind("unsupported", 0) == 0 ? SVM_E_UNSUPPORTED : SVM_E_INVALID_ARG,
                     "predication '" + t + "': " + err);
    collect_refs(pred, pred.root, &pred_refs);
  }
  // ---- joins: object k (1..n) joined at most once, on an int32 source column
  const int nref = (int)refs.size();
  if (nref > kMaxDims) return x->fail(SVM_E_UNSUPPORTED, "more than 4 joined objects");
  std::vector<int> join_of_obj(nref + 1, -1);
  for (size_t j = 0; j < b.join_rkey.size(); j++) {
    ColRef l = b.join_lkey[j], r = b.join_rkey[j];
    if (r.obj < 1 || r.obj > nref) return x->fail(SVM_E_INVALID_ARG, "rkey names an object the pipeline does not list");
    if (l.obj != 0) return x->fail(SVM_E_UNSUPPORTED, "lkey must be a column of the source object");
    if (join_of_obj[r.obj] >= 0) return x->fail(SVM_E_UNSUPPORTED, "an object joined twice");
    if (l.col < 0 || l.col >= src->ncols || r.col < 0 || r.col >= refs[r.obj - 1]->ncols)
      return x->fail(SVM_E_INVALID_ARG, "join column out of range");
    if (src->types[l.col] != SVM_INT32) return x->fail(SVM_E_UNSUPPORTED, "join keys must be int32");
    join_of_obj[r.obj] = (int)j;
  }
  for (auto& r : pred_refs)
    if (r.obj != 0)
      return x->fail(SVM_E_UNSUPPORTED, "a Filter on a joined object (the reference evaluates filters before joins)");
  // Operands: source columns (the projections' and conjuncts' own, then the
  // join keys), then joined columns as table payload fields.
  std::vector<ColRef> opnds;
  auto add_opnd = [&](const ColRef& r) {
    for (auto& o : opnds)
      if (o.obj == r.obj && o.col == r.col) return;
    opnds.push_back(r);
  };
  for (auto& r : refs_used)
    if (r.obj == 0) add_opnd(r);
  for (auto& r : pred_refs) add_opnd(r);
  for (auto& l : b.join_lkey) add_opnd(l);
  const int nfact = (int)opnds.size();
  std::vector<std::vector<int>> pay(nref + 1);
  for (auto& r : refs_used) {
    if (r.obj == 0) continue;
    if (r.obj > nref || join_of_obj[r.obj] < 0)
      return x->fail(SVM_E_INVALID_ARG, "Map references object " + std::to_string(r.obj) + " that is not joined");
    const ObjectPtr& o = refs[r.obj - 1];
    if (r.col < 0 || r.col >= o->ncols) return x->fail(SVM_E_INVALID_ARG, "column out of range");
    if (o->types[r.col] != SVM_INT32) return x->fail(SVM_E_UNSUPPORTED, "joined columns in a Map must be Int32");
    auto& v = pay[r.obj];
    if (std::find(v.begin(), v.end(), r.col) == v.end()) v.push_back(r.col);
  }
  for (int k = 1; k <= nref; k++) std::sort(pay[k].begin(), pay[k].end());
  for (int k = 1; k <= nref; k++)
    for (int c : pay[k]) add_opnd(ColRef{k, c});
  if (b.select_exp.size() > 16) return x->fail(SVM_E_UNSUPPORTED, "more than 16 projected columns");
  if (opnds.size() > 16) return x->fail(SVM_E_UNSUPPORTED, "more than 16 input columns referenced");
  for (int i = 0; i < nfact; i++) {
    const ColRef& r = opnds[i];
    if (r.col < 0 || r.col >= src->ncols) return x->fail(SVM_E_INVALID_ARG, "column out of range");
    // String columns are their int32 codes here: StrCmp tests were rewritten
    // onto them, and a bare projection copies them.
    if (src->types[r.col] != SVM_INT32 && src->types[r.col] != SVM_STRING)
      return x->fail(SVM_E_UNSUPPORTED, "only int32 and String input columns");
  }
  // A String output column is a bare String column of the source (StrCopy,
  // codegen/codegen.cpp:169-170).
  std::vector<int> str_src(b.select_exp.size(), -1);
  for (size_t i = 0; i < b.select_exp.size(); i++) {
    if (i >= b.sink.size()) return x->fail(SVM_E_INVALID_ARG, "Sink schema has fewer columns than the Map");
    const Node& root = proj[i].nodes[proj[i].root];
    const bool bare_str = root.kind == N_COL && src->is_string(root.ref.col);
    if (b.sink[i].type == SVM_STRING) {
      if (!bare_str) return x->fail(SVM_E_UNSUPPORTED, "a String output column must be a String input column");
      if (b.sink[i].val_size <= 0) return x->fail(SVM_E_INVALID_ARG, "a String output column needs a width");
      str_src[i] = root.ref.col;
    } else if (b.sink[i].type != SVM_INT32 || bare_str) {
      return x->fail(SVM_E_UNSUPPORTED, "projected columns must be declared Int32 (String for a String column)");
    }
  }
  SelectParams sp{};
  sp.ncols_in = nfact;
  sp.nopnd = (int)opnds.size();
  for (int k = 0; k < nfact; k++) sp.cols[k] = (const int32_t*)src->col(opnds[k].col);
  sp.nrows = (long long)src->nrows;
  sp.error = x->d_error;
  // ---- joined tables, probed in the order the joins are listed
  std::vector<DimTablePtr> tables;
  for (size_t j = 0; j < b.join_rkey.size(); j++) {
    const int k = b.join_rkey[j].obj;
    DimTablePtr T;
    svm_status st = build_dim(x, refs[k - 1], b.join_rkey[j].col, pay[k], &T);
    if (st) return st;
    tables.push_back(T);
    sp.dims[j] = T->desc;
    sp.dims[j].smem_word_off = -1;
    for (int i = 0; i < nfact; i++)
      if (opnds[i].obj == 0 && opnds[i].col == b.join_lkey[j].col) sp.join_opnd[j] = i;
  }
  sp.ndims = (int)tables.size();
  for (int i = nfact; i < sp.nopnd; i++) {
    const ColRef& r = opnds[i];
    const int d = join_of_obj[r.obj];
    const auto& pv = pay[r.obj];
    sp.dop[i - nfact] = Operand{(int8_t)d, (int8_t)(std::find(pv.begin(), pv.end(), r.col) - pv.begin())};
  }
  if (has_pred) {
    std::vector<int> conj;
    flatten_and(pred, pred.root, &conj);
    if (conj.size() <= 4) {
      for (int c : conj)
        if (!compile_prog(pred, c, opnds, &sp.pred[sp.npred++], &err)) return x->fail(SVM_E_UNSUPPORTED, err);
    } else if (!compile_prog(pred, pred.root, opnds, &sp.pred[sp.npred++], &err)) {
      return x->fail(SVM_E_UNSUPPORTED, err);
    }
  }
  sp.nout = (int)proj.size();
  for (size_t i = 0; i < proj.size(); i++)
    if (!compile_prog(proj[i], proj[i].root, opnds, &sp.proj[i], &err)) return x->fail(SVM_E_UNSUPPORTED, err);

  unsigned long long tiles = select_tiles(sp.nrows);
  x->scratch_reset();
  size_t need = 4 * (tiles + 1) + 8 * (tiles + 2) + 8 * scan_tmp_words(tiles) + 8 + 4096;
  svm_status st = x->scratch_reserve(need);
  if (st) return st;
  void *tc, *to, *tt, *b0;
  if ((st = x->scratch_take(4 * (tiles + 1), &tc)) || (st = x->scratch_take(8 * (tiles + 2), &to)) ||
      (st = x->scratch_take(8 * scan_tmp_words(tiles), &tt)) || (st = x->scratch_take(8, &b0)))
    return st;
  sp.tile_count = (unsigned int*)tc;
  sp.tile_offset = (unsigned long long*)to;
  sp.bulk0_count = (unsigned long long*)b0;
  sp.bulk0_rows = src->has_bulks ? (long long)src->bulk0_rows : 0;
  cudaError_t e = cudaMemsetAsync(b0, 0, 8, x->stream);
  cudaEvent_t ev;
  x->prof_begin(SVM_K_SELECT, &ev);
  if (!e) e = launch_select_count(sp, x->stream);
  if (!e) e = launch_exclusive_scan(sp.tile_count, tiles, (unsigned long long*)to, (unsigned long long*)tt, x->stream);
  x->prof_end(SVM_K_SELECT, ev);
  unsigned long long hdr[2] = {0, 0};
  if (!e) e = cudaMemcpyAsync(&hdr[0], (unsigned long long*)to + tiles, 8, cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaMemcpyAsync(&hdr[1], b0, 8, cudaMemcpyDeviceToHost, x->stream);
  if (e) return x->cuda_fail(e, "select count");
  if ((st = sync_and_check(x, "select count"))) return st;
  std::vector<int> types(proj.size(), SVM_INT32);
  ObjectPtr out = new_result_object(x, b.id, types, hdr[0], &st);
  if (st) return st;
  for (int o = 0; o < sp.nout; o++) sp.out[o] = (int32_t*)out->col(o);
  x->prof_begin(SVM_K_SELECT, &ev);
  e = launch_select_write(sp, x->stream);
  x->prof_end(SVM_K_SELECT, ev);
  if (e) return x->cuda_fail(e, "select write");
  // String outputs: the source's codes with its dictionary, or -- for a
  // narrower output column -- recoded into the dictionary of the cut values.
  // (A wider one is NUL-padded; the reference's StrCopy reads the next rows'
  // bytes there.)
  std::vector<DevBufPtr> luts;
  for (size_t i = 0; i < str_src.size(); i++) {
    if (str_src[i] < 0) continue;
    const StrCol& in = src->strs.at(str_src[i]);
    StrCol oc;
    oc.width = (int)b.sink[i].val_size;
    if (oc.width >= in.dict->width) {
      oc.dict = in.dict;
    } else {
      std::vector<int32_t> remap;
      oc.dict = truncate_dict(*in.dict, oc.width, &remap);
      DevBufPtr lut;
      if ((st = x->alloc(4 * remap.size() + 4, &lut))) return st;
      if (!e) e = cudaMemcpyAsync(lut->p, remap.data(), 4 * remap.size(), cudaMemcpyHostToDevice, x->stream);
      if (!e) e = launch_lut_gather((const int32_t*)out->col((int)i), out->nrows, (const int32_t*)lut->p,
                                    (int32_t*)out->col((int)i), x->stream);
      luts.push_back(lut);
    }
    out->types[i] = SVM_STRING;
    out->strs[(int)i] = oc;
  }
  if (e) return x->cuda_fail(e, "string recode");
  if ((st = sync_and_check(x, "select write"))) return st;
  // Output bulk i holds the rows of source bulk i (core/pipeline.cu:161-162, 289-332).
  out->has_bulks = src->has_bulks;
  out->bulk0_rows = hdr[1];
  out->source_rows = src->nrows;
  x->put_object(b.id, out);
  return SVM_OK;
}

// ============================================================ dimension tables
svm_status build_dim(Ctx* x, const ObjectPtr& obj, int key_col, const std::vector<int>& pay_cols,
                     DimTablePtr* out) {
  const bool compat = x->cfg.join_mode == SVM_JOIN_REF_COMPAT;
  const unsigned ht = (unsigned)(kHashRate * x->cfg.tuple_per_bulk);
  std::string key = obj->id + "#" + std::to_string(obj->version) + "#" + std::to_string(key_col) + "#";
  for (int c : pay_cols) key += std::to_string(c) + ",";
  key += compat ? "#ref" + std::to_string(ht) + (x->cfg.hash_char_signed ? "s" : "u") : "#exact";
  auto it = x->dim_cache.find(key);
  if (it != x->dim_cache.end()) {
    *out = it->second;
    return SVM_OK;
  }
  if (obj->types[key_col] != SVM_INT32) return x->fail(SVM_E_UNSUPPORTED, "join keys must be int32 columns");
  for (int c : pay_cols)
    if (obj->types[c] != SVM_INT32) return x->fail(SVM_E_UNSUPPORTED, "joined columns must be int32");
  if (pay_cols.size() > (size_t)(kMaxKeys + 2 * kMaxMetrics))
    return x->fail(SVM_E_UNSUPPORTED, "too many columns of one joined object");
  // REF_COMPAT: only bulk 0 of the joined object is probed (core/pipeline.cu:91, 295).
  long long n = compat ? (obj->has_bulks ? (long long)obj->bulk0_rows : 0) : (long long)obj->nrows;
  auto T = std::make_shared<DimTable>();
  T->rows_considered = (unsigned long long)n;
  T->pay_cols = pay_cols;

  BuildInput in{};
  in.key = (const int32_t*)obj->col(key_col);
  in.n = n;
  in.npay = (int)pay_cols.size();
  for (size_t f = 0; f < pay_cols.size(); f++) in.pay[f] = (const int32_t*)obj->col(pay_cols[f]);

  x->scratch_reset();
  size_t rc = compat && n > 0 ? refcompat_scratch_bytes(n, ht) : 0;
  size_t stats_words = 2 + 2 * pay_cols.size() + 1;
  svm_status st = x->scratch_reserve(rc + 4 * stats_words + 4096);
  if (st) return st;
  void *rcs = nullptr, *stats = nullptr;
  DevBufPtr dropped;  // REF_COMPAT: rows the reference's table leaves out
  if (rc && ((st = x->alloc((size_t)n, &dropped)) || (st = x->scratch_take(rc, &rcs)))) return st;
  if ((st = x->scratch_take(4 * stats_words, &stats))) return st;
  cudaError_t e = cudaSuccess;
  cudaEvent_t ev;
  x->prof_begin(SVM_K_BUILD, &ev);
  if (rc) {
    e = launch_refcompat(in.key, n, ht, x->cfg.hash_char_signed, (uint8_t*)dropped->p, rcs, x->stream);
    in.dropped = (const uint8_t*)dropped->p;
  }
  std::vector<int32_t> hs(stats_words);
  for (size_t f = 0; f < stats_words - 1; f += 2) {
    hs[f] = INT_MAX;
    hs[f + 1] = INT_MIN;
  }
  hs[stats_words - 1] = 0;
  if (!e) e = cudaMemcpyAsync(stats, hs.data(), 4 * stats_words, cudaMemcpyHostToDevice, x->stream);
  if (!e) e = launch_build_stats(in, (int32_t*)stats, x->stream);
  if (!e) e = cudaMemcpyAsync(hs.data(), stats, 4 * stats_words, cudaMemcpyDeviceToHost, x->stream);
  x->prof_end(SVM_K_BUILD, ev);
  if (e) return x->cuda_fail(e, "dimension stats");
  if ((st = sync_and_check(x, "dimension stats"))) return st;
  T->live = (uint32_t)hs[stats_words - 1];
  T->key_min = hs[0];
  T->key_max = hs[1];
  for (size_t f = 0; f < pay_cols.size(); f++) {
    T->pay_min.push_back(hs[2 + 2 * f]);
    T->pay_max.push_back(hs[3 + 2 * f]);
  }

  DimDesc& d = T->desc;
  d.smem_word_off = -1;
  d.npay = (int)pay_cols.size();
  if (T->live == 0) {
    // Nothing joinable: a dense table with an empty key range.
    d.layout = LAYOUT_DENSE;
    d.entry_bits = 1;
    d.key_min = 0;
    d.span = 0;
    d.table_words = 1;
    if ((st = x->alloc(4, &T->words, true))) return st;
    d.words = (const uint32_t*)T->words->p;
    for (int f = 0; f < d.npay; f++) d.pay[f] = PayloadField{nullptr, 0, 1, 0};
    x->dim_cache[key] = T;
    *out = T;
    return SVM_OK;
  }
  // Payload: bit-pack each column as (value - min) when the entry fits 32
  // bits, else store the row index and gather the columns at probe time.
  int bits_total = 1;
  std::vector<int> fbits(pay_cols.size());
  for (size_t f = 0; f < pay_cols.size(); f++) {
    unsigned long long range = (unsigned long long)((long long)T->pay_max[f] - T->pay_min[f] + 1);
    fbits[f] = ceil_log2(range);
    bits_total += fbits[f];
  }
  bool row_index = bits_total > 32;
  if (row_index) {
    int rb = ceil_log2((unsigned long long)n);
    bits_total = 1 + rb;
    for (size_t f = 0; f < pay_cols.size(); f++)
      d.pay[f] = PayloadField{(const int32_t*)obj->col(pay_cols[f]), 0, 1, (uint8_t)rb};
  } else {
    int shift = 1;
    for (size_t f = 0; f < pay_cols.size(); f++) {
      d.pay[f] = PayloadField{nullptr, T->pay_min[f], (uint8_t)shift, (uint8_t)fbits[f]};
      shift += fbits[f];
    }
  }
  int entry_bits = 1;
  while (entry_bits < bits_total) entry_bits <<= 1;
  unsigned long long span = (unsigned long long)((long long)T->key_max - T->key_min + 1);
  unsigned long long cap = 16;
  while (cap < 2 * T->live) cap <<= 1;
  unsigned long long dense_bytes = (span * entry_bits + 31) / 32 * 4;
  unsigned long long hash_bytes = cap * 8;
  // Dense when it is not much larger than the hash table would be; the
  // kernels index dense tables with 32-bit bit offsets.
  bool dense = span * (unsigned long long)entry_bits < (1ull << 32) &&
               dense_bytes <= std::max(2 * hash_bytes, 64ull << 10);
  d.key_min = T->key_min;
  x->scratch_reset();
  if (dense) {
    d.layout = LAYOUT_DENSE;
    d.entry_bits = entry_bits;
    d.span = (uint32_t)span;
    d.table_words = (uint32_t)(dense_bytes / 4);
    if ((st = x->alloc(dense_bytes, &T->words))) return st;
    d.words = (const uint32_t*)T->words->p;
    void* owner;
    if ((st = x->scratch_reserve(4 * span + 256)) || (st = x->scratch_take(4 * span, &owner))) return st;
    x->prof_begin(SVM_K_BUILD, &ev);
    e = launch_build_dense(in, d, (int32_t*)owner, (uint32_t*)T->words->p, x->stream);
    x->prof_end(SVM_K_BUILD, ev);
  } else {
    if (bits_total > 32) return x->fail(SVM_E_UNSUPPORTED, "joined payload too wide");
    d.layout = LAYOUT_HASH;
    d.entry_bits = 32;
    d.span = (uint32_t)cap;
    d.table_words = (uint32_t)(2 * cap);
    if ((st = x->alloc(hash_bytes, &T->words))) return st;
    d.words = (const uint32_t*)T->words->p;
    void* slots;
    size_t need = 8 * cap + 256;
    if ((st = x->scratch_reserve(need)) || (st = x->scratch_take(8 * cap, &slots))) return st;
    x->prof_begin(SVM_K_BUILD, &ev);
    e = launch_build_hash(in, d, (unsigned long long*)slots, (uint32_t*)T->words->p, x->d_error, x->stream);
    x->prof_end(SVM_K_BUILD, ev);
  }
  if (e) return x->cuda_fail(e, "dimension build");
  if ((st = sync_and_check(x, "dimension build"))) return st;
  x->dim_cache[key] = T;
  *out = T;
  return SVM_OK;
}

// ============================================================ star queries
struct StepPlan {
  Step step;
  double est;      // fraction of rows expected to survive the step
  int order_class; // 0 filter/probe, 1 plain load
};

// A planned fact pipeline: the kernel parameters (without scratch pointers)
// and the result object's shape.
struct StarPlan {
  StarParams P{};
  std::vector<int> fact_cols;   // StarParams::cols slot -> source column
  std::vector<int> out_types;
  int wide[kMaxMetrics] = {1, 1, 1};
  int nkeys = 0, nmet = 0;
  bool empty_src = false;       // the source has no bulk: empty result, no launch
  bool empty_filter = false;    // a contradictory filter: no row passes
  bool needs_prog = false;
  std::vector<DimTablePtr> dim_tables;  // per StarParams dim
  double est_pass = 1.0;        // expected fraction of rows passing every filter step
};

svm_status plan_star(Ctx* x, const Bound& b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs,
                     StarPlan* plan) {
  std::string err;
  const int nkeys = (int)b.reduce_key.size();
  const int nmet = (int)b.metric_exp.size();
  if (nkeys > kMaxKeys) return x->fail(SVM_E_UNSUPPORTED, "more than 3 ReduceBy dims (as the reference)");
  if (nmet < 1 || nmet > kMaxMetrics) return x->fail(SVM_E_UNSUPPORTED, "ReduceBy needs 1..3 metrics");
  if ((int)b.sink.size() < nkeys + nmet)
    return x->fail(SVM_E_INVALID_ARG, "Sink schema has fewer columns than dims + metrics");
  int wide[kMaxMetrics];
  for (int m = 0; m < nmet; m++) {
    int t = b.sink[nkeys + m].type;
    if (t != SVM_INT64 && t != SVM_INT32)
      return x->fail(SVM_E_UNSUPPORTED, "metric columns must be declared Int32 or Int64");
    wide[m] = t == SVM_INT64;
  }
  // ---- joins: object k (1..n) is joined at most once, on a fact column.
  const int nref = (int)refs.size();
  if (nref > kMaxDims) return x->fail(SVM_E_UNSUPPORTED, "more than 4 joined objects");
  std::vector<int> join_of_obj(nref + 1, -1);
  for (size_t j = 0; j < b.join_rkey.size(); j++) {
    ColRef l = b.join_lkey[j], r = b.join_rkey[j];
    if (r.obj < 1 || r.obj > nref) return x->fail(SVM_E_INVALID_ARG, "rkey names an object the pipeline does not list");
    if (l.obj != 0) return x->fail(SVM_E_UNSUPPORTED, "lkey must be a column of the source object");
    if (join_of_obj[r.obj] >= 0) return x->fail(SVM_E_UNSUPPORTED, "an object joined twice");
    if (l.col < 0 || l.col >= src->ncols || r.col < 0 || r.col >= refs[r.obj - 1]->ncols)
      return x->fail(SVM_E_INVALID_ARG, "join column out of range");
    if (src->types[l.col] != SVM_INT32) return x->fail(SVM_E_UNSUPPORTED, "join keys must be int32");
    join_of_obj[r.obj] = (int)j;
  }
  // ---- expressions
  Expr pred;
  bool has_pred = !b.filter_exp.empty();
  if (has_pred) {
    std::string t = join_filters(b.filter_exp);
    if (!parse_expr(t, &pred, &err))
      return x->fail(err.rfind("unsupported", 0) == 0 ? SVM_E_UNSUPPORTED : SVM_E_INVALID_ARG,
                     "predication '" + t + "': " + err);
  }
  std::vector<Expr> mexp(nmet);
  for (int m = 0; m < nmet; m++)
    if (!parse_expr(b.metric_exp[m], &mexp[m], &err))
      return x->fail(err.rfind("unsupported", 0) == 0 ? SVM_E_UNSUPPORTED : SVM_E_INVALID_ARG,
                     "metric '" + b.metric_exp[m] + "': " + err);
  // Column indices past ncols are derived columns (String keys' hash ranks);
  // String columns themselves appear only as the codes StrCmp tests read.
  auto check_ref = [&](const ColRef& r, bool allow_dims) -> svm_status {
    if (r.obj == 0) {
      if (r.col < 0 || r.col >= (int)src->types.size()) return x->fail(SVM_E_INVALID_ARG, "column out of range");
      if (src->types[r.col] != SVM_INT32 && src->types[r.col] != SVM_STRING)
        return x->fail(SVM_E_UNSUPPORTED, "only int32 fact columns");
      return SVM_OK;
    }
    if (!allow_dims)
      return x->fail(SVM_E_UNSUPPORTED, "a Filter on a joined object (the reference evaluates filters before joins)");
    if (r.obj > nref || join_of_obj[r.obj] < 0)
      return x->fail(SVM_E_INVALID_ARG, "reference to object " + std::to_string(r.obj) + " that is not joined");
    if (r.col < 0 || r.col >= (int)refs[r.obj - 1]->types.size())
      return x->fail(SVM_E_INVALID_ARG, "column out of range");
    return SVM_OK;
  };
  std::vector<ColRef> pred_refs, met_refs;
  if (has_pred) collect_refs(pred, pred.root, &pred_refs);
  for (auto& r : pred_refs)
    if (svm_status s = check_ref(r, false)) return s;
  for (int m = 0; m < nmet; m++) collect_refs(mexp[m], mexp[m].root, &met_refs);
  for (auto& r : met_refs)
    if (svm_status s = check_ref(r, true)) return s;
  for (auto& r : b.reduce_key)
    if (svm_status s = check_ref(r, true)) return s;

  // ---- the result object's shape
  std::vector<int> out_types(nkeys, SVM_INT32);
  for (int m = 0; m < nmet; m++) out_types.push_back(wide[m] ? SVM_INT64 : SVM_INT32);
  plan->out_types = out_types;
  plan->nkeys = nkeys;
  plan->nmet = nmet;
  for (int m = 0; m < nmet; m++) plan->wide[m] = wide[m];
  svm_status st;
  if (!src->has_bulks) {
    // No fact bulks: the reference runs no task and its sink stays empty.
    plan->empty_src = true;
    return SVM_OK;
  }

  // ---- filter conjuncts: ranges per fact column, the rest residual
  std::map<int, std::pair<int32_t, int32_t>> ranges;
  bool empty = false;
  std::vector<int> residual;
  if (has_pred) {
    std::vector<int> conj;
    flatten_and(pred, pred.root, &conj);
    for (int c : conj) {
      ColRef r;
      int32_t lo, hi, v;
      if (as_range(pred, c, &r, &lo, &hi)) {
        auto it = ranges.find(r.col);
        if (it == ranges.end()) {
          ranges[r.col] = {lo, hi};
        } else {
          it->second.first = std::max(it->second.first, lo);
          it->second.second = std::min(it->second.second, hi);
        }
        if (lo > hi) empty = true;
      } else if (const_value(pred, c, &v)) {
        if (!v) empty = true;
      } else {
        residual.push_back(c);
      }
    }
    for (auto& kv : ranges)
      if (kv.second.first > kv.second.second) empty = true;
  }

  // ---- dimension tables: payload = the joined object's columns used by keys/metrics
  std::vector<std::vector<int>> pay(nref + 1);
  auto add_pay = [&](const ColRef& r) {
    if (r.obj == 0) return;
    auto& v = pay[r.obj];
    if (std::find(v.begin(), v.end(), r.col) == v.end()) v.push_back(r.col);
  };
  for (auto& r : met_refs) add_pay(r);
  for (auto& r : b.reduce_key) add_pay(r);
  std::vector<DimTablePtr> tables(nref + 1);
  for (int k = 1; k <= nref; k++) {
    if (join_of_obj[k] < 0) continue;
    std::sort(pay[k].begin(), pay[k].end());
    st = build_dim(x, refs[k - 1], b.join_rkey[join_of_obj[k]].col, pay[k], &tables[k]);
    if (st) return st;
  }

  // ---- staged fact columns: every fact column the query reads
  StarParams& P = plan->P;
  P = StarParams{};
  P.error = x->d_error;
  P.wait_polls = x->wait_polls;
  P.stall_copies = x->stall_copies;
  P.row_begin = (long long)src->row0;
  P.row_end = (long long)(src->row0 + src->nrows);
  std::vector<int>& fact_cols = plan->fact_cols;  // StarParams::cols slot -> fact column
  auto col_slot = [&](int c) {
    for (size_t i = 0; i < fact_cols.size(); i++)
      if (fact_cols[i] == c) return (int)i;
    fact_cols.push_back(c);
    return (int)fact_cols.size() - 1;
  };
  std::vector<int> dim_of_obj(nref + 1, -1);
  int ndims = 0;
  for (int k = 1; k <= nref; k++)
    if (join_of_obj[k] >= 0) dim_of_obj[k] = ndims++;
  // ---- dims into StarParams, the smallest staged in shared memory
  P.ndims = ndims;
  std::vector<std::pair<size_t, int>> by_size;
  for (int k = 1; k <= nref; k++) {
    if (dim_of_obj[k] < 0) continue;
    P.dims[dim_of_obj[k]] = tables[k]->desc;
    P.dims[dim_of_obj[k]].smem_word_off = -1;
    by_size.push_back({(size_t)tables[k]->desc.table_words * 4, dim_of_obj[k]});
  }
  std::sort(by_size.begin(), by_size.end());
  int smem_words = 0;
  for (auto& bs : by_size) {
    if ((size_t)smem_words * 4 + bs.first > (size_t)kSmemTableBytes) break;
    P.dims[bs.second].smem_word_off = smem_words;
    smem_words += (int)((bs.first / 4 + 3) & ~size_t(3));
  }
  P.smem_table_words = smem_words;
  plan->dim_tables.assign(ndims, nullptr);
  for (int k = 1; k <= nref; k++)
    if (dim_of_obj[k] >= 0) plan->dim_tables[dim_of_obj[k]] = tables[k];
  // ---- filter steps: probes (a range on the same column folded in) and ranges
  struct StepPlan {
    Step step;
    double pass;   // expected fraction of rows that survive the step
    double cost;   // relative cost per row tested
  };
  auto range_pass = [&](int col, int32_t lo, int32_t hi, double* pass) -> svm_status {
    ColStats cs;
    svm_status s = x->column_stats(src, col, &cs);
    if (s) return s;
    double w = (double)cs.max - cs.min + 1;
    double ov = std::max(0.0, (double)std::min(cs.max, hi) - std::max(cs.min, lo) + 1);
    *pass = ov / w;
    return SVM_OK;
  };
  std::vector<StepPlan> order;
  std::set<int> ranged_done;
  for (int k = 1; k <= nref; k++) {
    if (join_of_obj[k] < 0) continue;
    int lc = b.join_lkey[join_of_obj[k]].col;
    StepPlan sp{};
    sp.step.kind = STEP_PROBE;
    sp.step.col = col_slot(lc);
    sp.step.lo = INT_MIN;
    sp.step.hi = INT_MAX;
    sp.step.dim = dim_of_obj[k];
    const DimTablePtr& T = tables[k];
    unsigned long long base_rows = std::max<unsigned long long>(1, refs[k - 1]->source_rows);
    sp.pass = std::min(1.0, (double)T->live / (double)base_rows);
    sp.cost = P.dims[sp.step.dim].smem_word_off >= 0 ? 1.0 : 4.0;
    auto r = ranges.find(lc);
    if (r != ranges.end()) {
      sp.step.lo = r->second.first;
      sp.step.hi = r->second.second;
      ranged_done.insert(lc);
      double rp;
      if ((st = range_pass(lc, r->second.first, r->second.second, &rp))) return st;
      sp.pass *= rp;
    }
    order.push_back(sp);
  }
  for (auto& kv : ranges) {
    if (ranged_done.count(kv.first)) continue;
    StepPlan sp{};
    sp.step.kind = STEP_RANGE;
    sp.step.col = col_slot(kv.first);
    sp.step.lo = kv.second.first;
    sp.step.hi = kv.second.second;
    sp.cost = 0.25;
    if ((st = range_pass(kv.first, kv.second.first, kv.second.second, &sp.pass))) return st;
    order.push_back(sp);
  }
  // Independent filters: ascending cost / (1 - pass) minimises the expected
  // work per row.
  std::stable_sort(order.begin(), order.end(), [](const StepPlan& a, const StepPlan& z) {
    return a.cost / std::max(1e-6, 1.0 - a.pass) < z.cost / std::max(1e-6, 1.0 - z.pass);
  });
  if ((int)order.size() > kMaxSteps) return x->fail(SVM_E_UNSUPPORTED, "more than 8 filter steps");
  P.nsteps = (int)order.size();
  plan->est_pass = 1.0;
  for (size_t s = 0; s < order.size(); s++) {
    P.steps[s] = order[s].step;
    plan->est_pass *= order[s].pass;
  }
  auto operand_of = [&](const ColRef& r, Operand* o) -> bool {
    if (r.obj == 0) {
      *o = Operand{(int8_t)col_slot(r.col), -1};
      return true;
    }
    int d = dim_of_obj[r.obj];
    if (d < 0) return false;
    auto& pv = pay[r.obj];
    int f = (int)(std::find(pv.begin(), pv.end(), r.col) - pv.begin());
    *o = Operand{(int8_t)d, (int8_t)f};
    return true;
  };
  // ---- operand table for bytecode programs
  std::vector<ColRef> prog_refs;
  auto add_prog_refs = [&](const Expr& e, int node) { collect_refs(e, node, &prog_refs); };
  for (int c : residual) add_prog_refs(pred, c);
  for (int m = 0; m < nmet; m++) add_prog_refs(mexp[m], mexp[m].root);
  if (prog_refs.size() > 16) return x->fail(SVM_E_UNSUPPORTED, "more than 16 columns in expressions");
  P.nopnd = (int)prog_refs.size();
  for (size_t i = 0; i < prog_refs.size(); i++)
    if (!operand_of(prog_refs[i], &P.opnds[i])) return x->fail(SVM_E_INVALID_ARG, "internal: unbound operand");
  if (residual.size() > (size_t)kMaxPost) return x->fail(SVM_E_UNSUPPORTED, "too many non-range filter terms");
  P.npost = (int)residual.size();
  for (size_t i = 0; i < residual.size(); i++)
    if (!compile_prog(pred, residual[i], prog_refs, &P.post[i], &err)) return x->fail(SVM_E_UNSUPPORTED, err);
  // ---- metrics
  P.nmetrics = nmet;
  for (int m = 0; m < nmet; m++) {
    Metric& M = P.metrics[m];
    const Node& root = mexp[m].nodes[mexp[m].root];
    if (root.kind == N_COL && operand_of(root.ref, &M.a)) {
      M.form = MF_OPND;
    } else if (root.kind == N_BINARY && (root.op == X_ADD || root.op == X_SUB || root.op == X_MUL) &&
               mexp[m].nodes[root.a].kind == N_COL && mexp[m].nodes[root.b].kind == N_COL &&
               operand_of(mexp[m].nodes[root.a].ref, &M.a) && operand_of(mexp[m].nodes[root.b].ref, &M.b)) {
      M.form = root.op == X_ADD ? MF_ADD : root.op == X_SUB ? MF_SUB : MF_MUL;
    } else {
      M.form = MF_PROG;
      if (!compile_prog(mexp[m], mexp[m].root, prog_refs, &M.prog, &err)) return x->fail(SVM_E_UNSUPPORTED, err);
    }
  }
  // ---- keys and the aggregation layout
  P.nkeys = nkeys;
  unsigned long long G = 1;
  for (int q = 0; q < nkeys; q++) {
    const ColRef& r = b.reduce_key[q];
    if (!operand_of(r, &P.keys[q])) return x->fail(SVM_E_INVALID_ARG, "internal: unbound key");
    int32_t lo, hi;
    if (r.obj == 0) {
      ColStats cs;
      if ((st = x->column_stats(src, r.col, &cs))) return st;
      lo = cs.min;
      hi = cs.max;
    } else {
      const DimTablePtr& T = tables[r.obj];
      auto& pv = pay[r.obj];
      int f = (int)(std::find(pv.begin(), pv.end(), r.col) - pv.begin());
      lo = T->live ? T->pay_min[f] : 0;
      hi = T->live ? T->pay_max[f] : 0;
    }
    if (hi < lo) hi = lo;
    P.kmin[q] = lo;
    P.krange[q] = (uint32_t)std::min<long long>((long long)hi - lo + 1, 0xFFFFFFFFll);
    if ((long long)hi - lo + 1 > (1ll << 26) || G * P.krange[q] > (1ull << 26))
      return x->fail(SVM_E_UNSUPPORTED, "group-key space above 2^26 groups (hash aggregation not built)");
    G *= P.krange[q];
  }
  unsigned long long stride = 1;
  for (int q = nkeys - 1; q >= 0; q--) {
    P.kstride[q] = stride;
    stride *= P.krange[q];
  }
  P.ngroups = G;
  if (nkeys == 0)
    P.agg = AGG_SCALAR;
  else if (G * (8ull * nmet + 4) <= (unsigned long long)kSmemAggBytes)
    P.agg = AGG_DENSE_SMEM;
  else
    P.agg = AGG_DENSE_GLOBAL;

  if ((int)fact_cols.size() > kMaxSteps) return x->fail(SVM_E_UNSUPPORTED, "query reads more than 8 fact columns");
  P.ncols = (int)fact_cols.size();
  for (size_t i = 0; i < fact_cols.size(); i++) P.cols[i] = (const int32_t*)src->base(fact_cols[i]);
  plan->empty_filter = empty;
  plan->needs_prog = P.npost > 0;
  for (int m = 0; m < nmet; m++) plan->needs_prog |= P.metrics[m].form == MF_PROG;
  flatten_plan(P);
  return SVM_OK;
}

// ---- plan cache
// A server sees the same query text again and again (under new pipeline
// ids); planning it -- parsing, column statistics, table lookups, the step
// order -- is most of the host time per request.  Plans are kept by the
// bound pipeline's content (after String rewriting, id excluded) and the
// identity, version and row range of every object it reads, so a replaced
// or regenerated object never meets a stale plan; the plans that read an
// object are forgotten when it is dropped or replaced.
struct PlanCache {
  std::unordered_map<std::string, StarPlan> plans;
  std::unordered_map<const Object*, std::vector<std::string>> by_object;
};

PlanCache* plan_cache(Ctx* x) {
  if (!x->plan_cache) x->plan_cache = std::make_shared<PlanCache>();
  return static_cast<PlanCache*>(x->plan_cache.get());
}

std::string plan_key(const Bound& b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs) {
  std::string k;
  auto add = [&](const std::string& t) {
    k += t;
    k += '\x1f';
  };
  for (auto& e : b.filter_exp) add(e);
  k += '\x1e';
  for (auto& e : b.metric_exp) add(e);
  k += '\x1e';
  for (auto* v : {&b.reduce_key, &b.join_lkey, &b.join_rkey}) {
    for (auto& r : *v) add(std::to_string(r.obj) + "." + std::to_string(r.col));
    k += '\x1e';
  }
  for (auto& c : b.sink) add(std::to_string(c.type) + ":" + std::to_string(c.val_size));
  k += '\x1e';
  auto obj = [&](const ObjectPtr& o) {
    add(std::to_string((uintptr_t)o.get()) + ":" + std::to_string(o->version) + ":" + std::to_string(o->row0) + ":" +
        std::to_string(o->nrows));
  };
  obj(src);
  for (auto& r : refs) obj(r);
  return k;
}

svm_status plan_star_cached(Ctx* x, const Bound& b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs,
                            StarPlan* plan) {
  PlanCache* pc = plan_cache(x);
  const std::string key = plan_key(b, src, refs);
  auto hit = pc->plans.find(key);
  if (hit != pc->plans.end()) {
    *plan = hit->second;
    plan->P.error = x->d_error;
    plan->P.wait_polls = x->wait_polls;
    plan->P.stall_copies = x->stall_copies;
    return SVM_OK;
  }
  svm_status st = plan_star(x, b, src, refs, plan);
  if (st) return st;
  if (pc->plans.size() >= 4096) {
    pc->plans.clear();
    pc->by_object.clear();
  }
  pc->plans.emplace(key, *plan);
  pc->by_object[src.get()].push_back(key);
  for (auto& r : refs) pc->by_object[r.get()].push_back(key);
  return SVM_OK;
}

// Presence prefilter (single-query scans).  A selective join whose dense
// table carries a payload and is too big to stage -- the part table of the
// date + part query: 400 K one-byte entries probed in L2 by every fact row,
// 4 % of them present -- gets a second, payload-less table over the same
// keys (one bit a key, the same rows inserted, so REF_COMPAT drops the same
// keys): its probe takes the payload probe's place, and the payload probe
// moves behind every other step, where only surviving rows reach it.  The
// bit table is small enough to stay in L1 or in shared memory.
svm_status add_presence_prefilters(Ctx* x, const Bound& b, const std::vector<ObjectPtr>& refs, StarPlan* plan) {
  StarParams& P = plan->P;
  if (plan->empty_src || plan->needs_prog) return SVM_OK;
  const int nref = (int)refs.size();
  std::vector<int> dim_obj;  // dim index -> joined object (1..nref), as plan_star numbers them
  std::vector<int> key_col;
  for (int k = 1; k <= nref; k++)
    for (size_t j = 0; j < b.join_rkey.size(); j++)
      if (b.join_rkey[j].obj == k) {
        dim_obj.push_back(k);
        key_col.push_back(b.join_rkey[j].col);
      }
  if ((int)dim_obj.size() != P.ndims) return SVM_OK;
  const int ndims0 = P.ndims;
  bool done[kMaxDims] = {};
  for (int s = 0; s < P.nsteps && P.ndims < kMaxDims && P.nsteps < kMaxSteps; s++) {
    const Step st = P.steps[s];
    if (st.kind != STEP_PROBE || st.dim >= ndims0 || done[st.dim]) continue;
    const DimDesc& D = P.dims[st.dim];
    if (D.layout != LAYOUT_DENSE || D.smem_word_off >= 0 || D.entry_bits < 2) continue;
    const DimTablePtr& T = plan->dim_tables[st.dim];
    const ObjectPtr& o = refs[dim_obj[st.dim] - 1];
    const double pass = (double)T->live / (double)std::max<unsigned long long>(1, o->source_rows);
    if (pass > 0.1 || (unsigned long long)D.span / 8 > (unsigned long long)kSmemTableBytes) continue;
    DimTablePtr pres;
    svm_status r = build_dim(x, o, key_col[st.dim], {}, &pres);
    if (r) return r;
    if (pres->desc.layout != LAYOUT_DENSE || pres->desc.entry_bits != 1) continue;
    done[st.dim] = true;
    const int nd = P.ndims++;
    P.dims[nd] = pres->desc;
    P.dims[nd].smem_word_off = -1;
    const int words = (int)((pres->desc.table_words + 3) & ~3u);
    if (P.smem_table_words + words <= kSmemTableBytes / 4) {  // staged when it fits beside the others
      P.dims[nd].smem_word_off = P.smem_table_words;
      P.smem_table_words += words;
    }
    plan->dim_tables.push_back(pres);
    // the bit probe (with any folded key range) in place of the payload probe,
    // which moves behind every other step
    Step bit = st;
    bit.dim = nd;
    Step payload = st;
    payload.lo = INT_MIN;
    payload.hi = INT_MAX;
    for (int k = s; k + 1 < P.nsteps; k++) P.steps[k] = P.steps[k + 1];
    P.steps[P.nsteps - 1] = payload;
    for (int k = P.nsteps; k > s; k--) P.steps[k] = P.steps[k - 1];
    P.steps[s] = bit;
    P.nsteps++;
  }
  flatten_plan(P);
  return SVM_OK;
}

// The shape a star launch is tuned for: columns, steps (kind, table layout,
// placement, entry width), dimensions, aggregation, and the orders of
// magnitude of the group count and the rows scanned.
std::string star_shape_key(const StarParams& P) {
  auto lg = [](unsigned long long v) {
    int b = 0;
    while (v > 1) {
      v >>= 1;
      b++;
    }
    return b;
  };
  std::string k = std::to_string(P.ncols) + ":" + std::to_string(P.ndims) + ":" + std::to_string(P.agg) + ":" +
                  std::to_string(P.nkeys) + ":" + std::to_string(P.nmetrics) + ":" + std::to_string(P.npost) + ":" +
                  std::to_string(lg(P.ngroups)) + ":" +
                  std::to_string(lg((unsigned long long)(P.row_end - P.row_begin) + 1)) + ":" +
                  std::to_string(P.agg_words) + "|";
  for (int i = 0; i < P.nsteps; i++) {
    const Step& st = P.steps[i];
    const DimDesc* D = st.kind == STEP_PROBE ? &P.dims[st.dim] : nullptr;
    k += std::to_string(st.kind) + (D ? "," + std::to_string(D->layout) + "," +
                                            std::to_string(D->smem_word_off >= 0) + "," +
                                            std::to_string(D->entry_bits) + "," + std::to_string(lg(D->span))
                                      : std::string()) + ";";
  }
  return k;
}

// Hash-rank keys back to the reference's Hash values (ranks order like the
// hashes, so the rows stay sorted by key).
svm_status translate_keys(Ctx* x, const Bound& b, const ObjectPtr& out) {
  cudaError_t e = cudaSuccess;
  std::vector<DevBufPtr> luts;
  for (size_t q = 0; q < b.key_hash.size(); q++) {
    if (b.key_hash[q].empty() || out->nrows == 0) continue;
    DevBufPtr lut;
    svm_status st = x->alloc(4 * b.key_hash[q].size(), &lut);
    if (st) return st;
    if (!e) e = cudaMemcpyAsync(lut->p, b.key_hash[q].data(), 4 * b.key_hash[q].size(), cudaMemcpyHostToDevice,
                                x->stream);
    if (!e) e = launch_lut_gather((const int32_t*)out->col((int)q), out->nrows, (const int32_t*)lut->p,
                                  (int32_t*)out->col((int)q), x->stream);
    luts.push_back(lut);
  }
  if (e) return x->cuda_fail(e, "string key translation");
  return luts.empty() ? SVM_OK : sync_and_check(x, "string key translation");
}

svm_status run_star(Ctx* x, const Bound& b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs) {
  StarPlan plan;
  svm_status st = plan_star_cached(x, b, src, refs, &plan);
  if (st) return st;
  if ((st = add_presence_prefilters(x, b, refs, &plan))) return st;
  const std::vector<int>& out_types = plan.out_types;
  const int nkeys = plan.nkeys, nmet = plan.nmet;
  const int* wide = plan.wide;
  if (plan.empty_src) {
    ObjectPtr out = new_result_object(x, b.id, out_types, 0, &st);
    if (st) return st;
    x->put_object(b.id, out);
    return SVM_OK;
  }
  StarParams& P = plan.P;
  const unsigned long long G = P.ngroups;
  const bool empty = plan.empty_filter;

  // ---- scratch: sums + counts (+ finalize buffers)
  x->scratch_reset();
  size_t agg_bytes = 8 * (size_t)G * (nmet + 1);
  size_t fin_bytes = nkeys ? 8 * ((G + 1) / 2 + 1 + G + 1) + 8 * scan_tmp_words(G) : 0;
  if ((st = x->scratch_reserve(agg_bytes + fin_bytes + 4096))) return st;
  void *sums, *fin = nullptr, *scant = nullptr;
  if ((st = x->scratch_take(agg_bytes, &sums))) return st;
  if (nkeys && ((st = x->scratch_take(8 * ((G + 1) / 2 + 1 + G + 1), &fin)) ||
                (st = x->scratch_take(8 * scan_tmp_words(G), &scant))))
    return st;
  P.sums = (unsigned long long*)sums;
  P.counts = P.sums + (size_t)nmet * G;
  cudaError_t e = cudaMemsetAsync(sums, 0, agg_bytes, x->stream);
  if (e) return x->cuda_fail(e, "cudaMemsetAsync");
  if (empty) P.row_end = P.row_begin;  // a contradictory filter: no row can pass

  // Launch configuration: the kernel (compiled for the plan's shape with 4
  // or 8 rows per consumer lane, or the interpreted kernel), ring depth and
  // whether the small dimension tables are staged in shared memory.  The
  // rule: a compiled kernel with 4 rows per lane when the shape has one, then
  // the most resident blocks per SM, the deepest ring, tables staged.  With
  // autotuning, every fitting candidate is timed once per plan shape on the
  // query itself (each trial starts from zeroed slots, so the result is the
  // same whichever wins), and also the order of two adjacent probes of
  // tables kept in L2 (filters commute; their relative cost depends on the
  // tables' sizes).
  using Cand = Ctx::StarLaunch;
  std::vector<int> staged_off(P.ndims);
  for (int d = 0; d < P.ndims; d++) staged_off[d] = P.dims[d].smem_word_off;
  const int staged_words = P.smem_table_words;
  bool any_staged = false;
  for (int d = 0; d < P.ndims; d++) any_staged |= staged_off[d] >= 0;
  const std::vector<Step> steps0(P.steps, P.steps + P.nsteps);
  const std::string shape = x->cfg.autotune ? star_shape_key(P) + "|pin" + std::to_string(x->pin_rows) + "," +
                                                 std::to_string(x->pin_minb) + "," + std::to_string(x->pin_stages) +
                                                 "," + std::to_string(x->pin_staged) + "," +
                                                 std::to_string(x->pin_list)
                                           : std::string();  // as planned
  // The compiled kernel reads the columns no filter step needs only at the
  // surviving rows (late columns); the interpreted kernel stages them all.
  // For a host-resident fact table the staged columns are device copies
  // (host_to_dev) and the late columns stay in host memory.
  const StarParams P0 = P;
  std::map<const int32_t*, const int32_t*> host_to_dev;
  bool host_unmapped = false;  // a staged column still points at host memory
  auto configure = [&](const Cand& c) {
    P = P0;
    P.nstages = c.nst;
    for (int d = 0; d < P.ndims; d++) P.dims[d].smem_word_off = c.staged ? staged_off[d] : -1;
    P.smem_table_words = c.staged ? staged_words : 0;
    for (int k = 0; k < P.nsteps; k++) P.steps[k] = steps0[k];
    if (c.swap >= 0) std::swap(P.steps[c.swap], P.steps[c.swap + 1]);
    if (c.rows) apply_late_columns(P);
    flatten_plan(P);
    host_unmapped = false;
    P.host_late = src->host ? 1 : 0;
    if (src->host)
      for (int k = 0; k < P.ncols; k++) {
        auto it = host_to_dev.find(P.cols[k]);
        if (it != host_to_dev.end())
          P.cols[k] = it->second;
        else
          host_unmapped = true;
      }
  };
  auto smem_of = [&](const Cand& c) { return c.rows ? star_plan_smem_bytes(P, c.rows) : star_smem_bytes(P); };
  auto grid_of = [&](const Cand& c, size_t sm) {
    return c.rows ? star_plan_grid_size(P, c.rows, c.minb, c.list, sm) : star_grid_size(P, sm);
  };
  auto launch = [&](const Cand& c, size_t sm) {
    if (host_unmapped) return cudaErrorInvalidValue;  // never scan host memory with bulk copies
    return c.rows ? launch_star_plan(P, c.rows, c.minb, c.list, grid_of(c, sm), sm, x->stream)
                  : launch_star(P, grid_of(c, sm), star_block_size(), sm, x->stream);
  };
  std::vector<int> swaps = {-1};
  if (x->cfg.autotune)
    for (int k = 0; k + 1 < P.nsteps; k++) {
      const Step &a = steps0[k], &z = steps0[k + 1];
      if (a.kind == STEP_PROBE && z.kind == STEP_PROBE && staged_off[a.dim] < 0 && staged_off[z.dim] < 0)
        swaps.push_back(k);
    }
  struct Fit {
    Cand c;
    int blocks;
  };
  std::vector<Fit> cands;
  for (int sw : swaps)
    for (int staged = 1; staged >= (any_staged ? 0 : 1); staged--)
      for (const auto& rm : {std::make_pair(4, 3), std::make_pair(4, 4), std::make_pair(8, 2), std::make_pair(0, 0)})
        for (int nst = kStages; nst >= 2; nst--)
          for (int la = 4; la >= 0; la--) {
            const int rows = rm.first;
            if ((x->pin_rows >= 0 && rows != x->pin_rows) || (x->pin_stages && nst != x->pin_stages) ||
                (x->pin_staged >= 0 && staged != x->pin_staged) || (x->pin_minb && rm.second != x->pin_minb) ||
                (x->pin_list >= 0 && la != x->pin_list) || (!rows && la != 3))
              continue;
            Cand c;
            c.nst = nst;
            c.staged = staged != 0;
            c.swap = sw;
            c.rows = rows;
            c.minb = rm.second;
            c.list = la;
            configure(c);
            if (rows && !star_plan_available(P, rows, c.minb, la)) continue;
            const size_t sm = smem_of(c);
            if (sm > 200 * 1024) continue;
            const int blocks = rows ? star_plan_blocks_per_sm(P, rows, c.minb, la, sm) : star_blocks_per_sm(P, sm);
            // a kernel built for 4 blocks per SM where fewer fit gains nothing over the one built for 3
            if (blocks > 0 && !(rows && c.minb > 3 && blocks < c.minb)) cands.push_back({c, blocks});
          }
  if (cands.empty())
    return x->fail(SVM_E_UNSUPPORTED, x->pin_rows >= 0 || x->pin_minb || x->pin_stages || x->pin_staged >= 0 ||
                                              x->pin_list >= 0
                                          ? "no launch configuration of this plan fits the pinned choices"
                                          : "shared-memory plan too large");
  // A host-resident fact table: every candidate must stage the same columns,
  // so only compiled kernels run its scan when one fits (they all keep the
  // same late columns); the staged columns' rows this scan reads are copied
  // to the device now, the late ones are gathered from host memory.  (The
  // gathers cross the same host link as the copies, about one transfer per
  // surviving row; overlapping the copies with the scan in row chunks was
  // measured and gains nothing: the link's bytes bound both.)
  std::vector<DevBufPtr> host_copies;
  if (src->host) {
    bool any_compiled = false;
    for (const Fit& f : cands) any_compiled |= f.c.rows != 0;
    if (any_compiled)
      cands.erase(std::remove_if(cands.begin(), cands.end(), [](const Fit& f) { return f.c.rows == 0; }),
                  cands.end());
    configure(cands[0].c);
    const long long a0 = P.row_begin & ~3ll, end4 = (P.row_end + 3) & ~3ll;
    for (int k = 0; k < P.ncols; k++) {
      const int32_t* h = P.cols[k];
      if (host_to_dev.count(h)) continue;
      const DevBuf* hb = nullptr;
      int hk = -1;
      for (size_t s = 0; s < src->storage.size(); s++)
        if (src->storage[s] && src->storage[s]->p == (const void*)h) {
          hb = src->storage[s].get();
          hk = (int)s;
        }
      if (!h || !hb) return x->fail(SVM_E_INVALID_ARG, "a host-resident column the scan reads has no data");
      auto dc = src->dev_copy.find(hk);
      if (dc != src->dev_copy.end() && dc->second) {  // copied already, for its statistics
        host_to_dev[h] = (const int32_t*)dc->second->p;
        continue;
      }
      const long long base_rows = (long long)(hb->bytes / 4);
      const long long hi = std::min(end4, base_rows);
      DevBufPtr d;
      if ((st = x->alloc((size_t)(end4 - a0 + 64) * 4, &d))) return st;
      if (hi > a0 && (e = cudaMemcpyAsync(d->p, h + a0, (size_t)(hi - a0) * 4, cudaMemcpyHostToDevice, x->stream)))
        return x->cuda_fail(e, "host-resident column copy");
      host_to_dev[h] = (const int32_t*)d->p - a0;  // indexed by base row, like the host column
      host_copies.push_back(d);
    }
  }
  auto same_cand = [](const Cand& a, const Cand& z) {
    return a.nst == z.nst && a.staged == z.staged && a.swap == z.swap && a.rows == z.rows && a.minb == z.minb &&
           a.list == z.list;
  };
  auto rule_rank = [](const Fit& f) {  // larger is preferred
    return (f.c.rows == 4 ? 2 : f.c.rows == 8 ? 1 : 0) * 10000000 + (f.c.list == 3 ? 1000000 : 0) +
           f.blocks * 1000 + f.c.nst * 10 + (f.c.staged ? 1 : 0);
  };
  Cand pick = cands[0].c;
  int best_rank = -1;
  for (const Fit& f : cands)
    if (f.c.swap < 0 && rule_rank(f) > best_rank) {
      best_rank = rule_rank(f);
      pick = f.c;
    }
  cudaEvent_t ev;
  if (x->cfg.autotune && cands.size() > 1) {
    const std::string& key = shape;
    auto hit = x->star_tune.find(key);
    if (hit != x->star_tune.end()) {
      pick = hit->second;
    } else if (!src->host) {  // a host-resident table takes the cached choice or the rule
      cudaEvent_t t0, t1;
      cudaEventCreate(&t0);
      cudaEventCreate(&t1);
      float best = 0.f;
      for (const Fit& f : cands) {
        configure(f.c);
        // Candidates are ranked on the first kTuneRows rows of the scan (the
        // query itself then runs whole with the pick), so that the first run
        // of a shape costs tens of milliseconds, not a full scan per candidate.
        constexpr long long kTuneRows = 1ll << 25;
        if (P.row_end - P.row_begin > kTuneRows) P.row_end = P.row_begin + kTuneRows;
        const size_t sm = smem_of(f.c);
        if (!e) e = cudaMemsetAsync(sums, 0, agg_bytes, x->stream);
        if (!e) e = cudaEventRecord(t0, x->stream);
        if (!e) e = launch(f.c, sm);
        if (!e) e = cudaEventRecord(t1, x->stream);
        if (!e) e = cudaEventSynchronize(t1);
        float ms = 0.f;
        if (!e) e = cudaEventElapsedTime(&ms, t0, t1);
        if (e) break;
        if (best == 0.f || ms < best) {
          best = ms;
          pick = f.c;
        }
      }
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
      if (e) return x->cuda_fail(e, "star kernel tuning");
      x->star_tune[key] = pick;
      if ((e = cudaMemsetAsync(sums, 0, agg_bytes, x->stream))) return x->cuda_fail(e, "cudaMemsetAsync");
    }
  }
  if (src->host) {  // a choice cached from a device-resident table may not stage the same columns
    bool ok = false;
    for (const Fit& f : cands) ok |= same_cand(f.c, pick);
    if (!ok) {
      int r = -1;
      for (const Fit& f : cands)
        if (rule_rank(f) > r) {
          r = rule_rank(f);
          pick = f.c;
        }
    }
  }
  configure(pick);
  size_t smem = smem_of(pick);
  int grid = grid_of(pick, smem);
  const int resident = pick.rows ? star_plan_blocks_per_sm(P, pick.rows, pick.minb, pick.list, smem)
                                 : star_blocks_per_sm(P, smem);
  {
    std::string steps;
    for (int k = 0; k < P.nsteps; k++) {
      const Step& st = P.steps[k];
      steps += (k ? "," : "") + std::string(st.kind == STEP_RANGE ? "range" : st.layout == LAYOUT_HASH ? "hash"
                                                                     : st.smem_word_off >= 0 ? "smem"
                                                                                             : "l2");
      if (st.kind == STEP_PROBE && st.layout == LAYOUT_DENSE) steps += std::to_string(st.entry_bits);
    }
    x->last_launch = std::string("{\"kernel\": \"") + (pick.rows ? "compiled plan" : "interpreted") +
                     "\", \"rows_per_lane\": " + std::to_string(pick.rows ? pick.rows : 4) +
                     ", \"blocks_per_sm_compiled_for\": " + std::to_string(pick.minb ? pick.minb : 3) +
                     ", \"blocks_per_sm\": " + std::to_string(resident) +
                     ", \"list_after_step\": " + std::to_string(pick.rows ? pick.list : 3) +
                     ", \"ring_stages\": " + std::to_string(pick.nst) + ", \"tables_staged\": " +
                     (pick.staged ? "true" : "false") + ", \"steps\": \"" + steps + "\", \"grid\": " +
                     std::to_string(grid) + ", \"block\": " + std::to_string(star_block_size()) +
                     ", \"smem_bytes\": " + std::to_string(smem) + ", \"staged_columns\": " +
                     std::to_string(P.ncols) + ", \"late_columns\": " + std::to_string(P.nlate) + ", \"tuned\": " +
                     (x->cfg.autotune && cands.size() > 1 ? "true" : "false") + "}";
  }
  x->prof_begin(SVM_K_STAR, &ev);
  e = launch(pick, smem);
  x->prof_end(SVM_K_STAR, ev);
  if (e) return x->cuda_fail(e, "star kernel");

  ObjectPtr out;
  if (nkeys == 0) {
    std::vector<unsigned long long> h(nmet);
    e = cudaMemcpyAsync(h.data(), sums, 8 * nmet, cudaMemcpyDeviceToHost, x->stream);
    if (e) return x->cuda_fail(e, "result copy");
    if ((st = sync_and_check(x, "star query"))) return st;
    out = new_result_object(x, b.id, out_types, 1, &st);
    if (st) return st;
    for (int m = 0; m < nmet; m++) {
      if (wide[m]) {
        long long v = (long long)h[m];
        e = cudaMemcpyAsync(out->col(m), &v, 8, cudaMemcpyHostToDevice, x->stream);
      } else {
        int32_t v = (int32_t)(uint32_t)h[m];
        e = cudaMemcpyAsync(out->col(m), &v, 4, cudaMemcpyHostToDevice, x->stream);
      }
      if (!e) e = cudaStreamSynchronize(x->stream);
      if (e) return x->cuda_fail(e, "result store");
    }
  } else {
    x->prof_begin(SVM_K_FINALIZE, &ev);
    e = launch_finalize_dense(P, nullptr, nullptr, nullptr, (unsigned long long*)fin,
                              (unsigned long long*)scant, nullptr, x->stream);
    x->prof_end(SVM_K_FINALIZE, ev);
    unsigned long long ng = 0;
    unsigned long long* pos = (unsigned long long*)fin + (G + 1) / 2 + 1;
    if (!e) e = cudaMemcpyAsync(&ng, pos + G, 8, cudaMemcpyDeviceToHost, x->stream);
    if (e) return x->cuda_fail(e, "finalize");
    if ((st = sync_and_check(x, "star query"))) return st;
    out = new_result_object(x, b.id, out_types, ng, &st);
    if (st) return st;
    int32_t* kout[kMaxKeys];
    void* mout[kMaxMetrics];
    for (int q = 0; q < nkeys; q++) kout[q] = (int32_t*)out->col(q);
    for (int m = 0; m < nmet; m++) mout[m] = out->col(nkeys + m);
    x->prof_begin(SVM_K_FINALIZE, &ev);
    e = launch_finalize_dense(P, kout, mout, wide, (unsigned long long*)fin, (unsigned long long*)scant,
                              nullptr, x->stream);
    x->prof_end(SVM_K_FINALIZE, ev);
    if (e) return x->cuda_fail(e, "finalize write");
    if ((st = sync_and_check(x, "finalize"))) return st;
    if ((st = translate_keys(x, b, out))) return st;
  }
  out->has_bulks = true;
  out->bulk0_rows = out->nrows;
  x->put_object(b.id, out);
  return SVM_OK;
}

}  // namespace

namespace {

// The derived column of object o's String column c holding each row's rank
// among the Hash values of the codes its storage holds.  It is computed once
// per code storage over the storage's whole extent (its zeroed padding rows
// hold code 0), so views of an object share it and a batched union scan over
// several views' ranges stays inside it.
svm_status ensure_rank_col(Ctx* x, const ObjectPtr& o, int c, int* idx) {
  StrCol& sc = o->strs.at(c);
  if (sc.rank_col >= 0) {
    *idx = sc.rank_col;
    return SVM_OK;
  }
  const DevBufPtr& codes = o->storage[c];
  const auto key = std::make_tuple((const void*)codes.get(), (const void*)sc.dict.get(), sc.width);
  auto it = x->rank_cache.find(key);
  if (it == x->rank_cache.end()) {
    const unsigned long long rows = codes->bytes / 4;
    const uint32_t D = sc.dict->count;
    std::vector<uint32_t> present(D, 0);
    DevBufPtr flags, lut, ranks;
    svm_status st;
    if ((st = x->alloc(4ull * D + 4, &flags, true))) return st;
    cudaError_t e = launch_mark_codes((const int32_t*)codes->p, rows, (uint32_t*)flags->p, x->stream);
    if (!e && D) e = cudaMemcpyAsync(present.data(), flags->p, 4ull * D, cudaMemcpyDeviceToHost, x->stream);
    if (!e) e = cudaStreamSynchronize(x->stream);
    if (e) return x->cuda_fail(e, "string key codes");
    Ctx::RankCol rc;
    std::vector<int32_t> rank_of_code;
    hash_ranks(*sc.dict, sc.width, present, &rank_of_code, &rc.hash_of_rank);
    if ((st = x->alloc(4 * rank_of_code.size() + 4, &lut)) || (st = x->alloc(4 * rows, &ranks, true))) return st;
    e = cudaMemcpyAsync(lut->p, rank_of_code.data(), 4 * rank_of_code.size(), cudaMemcpyHostToDevice, x->stream);
    if (!e) e = launch_lut_gather((const int32_t*)codes->p, rows, (const int32_t*)lut->p, (int32_t*)ranks->p,
                                  x->stream);
    if (e) return x->cuda_fail(e, "string key ranks");
    if ((st = sync_and_check(x, "string key ranks"))) return st;
    rc.codes = codes;
    rc.ranks = ranks;
    it = x->rank_cache.emplace(key, std::move(rc)).first;
  }
  o->types.push_back(SVM_INT32);
  o->storage.push_back(it->second.ranks);
  if (o->stats.size() < o->types.size()) o->stats.resize(o->types.size());
  const int32_t h = (int32_t)it->second.hash_of_rank.size();
  o->stats.back() = ColStats{true, 0, h > 0 ? h - 1 : 0};
  sc.rank_col = (int)o->types.size() - 1;
  sc.rank_hash = it->second.hash_of_rank;
  *idx = sc.rank_col;
  return SVM_OK;
}

// String columns in a bound pipeline: StrCmp comparisons in Filter, Map and
// metric expressions become tests of the codes; String ReduceBy keys become
// their hash-rank columns (b->key_hash keeps the way back); String join keys
// and any other use of a String column are unsupported.
svm_status resolve_strings(Ctx* x, Bound* b, const ObjectPtr& src, const std::vector<ObjectPtr>& refs) {
  // Nothing to do without String columns or StrCmp (no parsing on the common path).
  bool any = !src->strs.empty();
  for (const ObjectPtr& r : refs) any |= !r->strs.empty();
  for (const auto* v : {&b->filter_exp, &b->metric_exp, &b->select_exp})
    for (const std::string& t : *v) any |= t.find("StrCmp") != std::string::npos;
  b->key_hash.assign(b->reduce_key.size(), {});
  if (!any) return SVM_OK;
  auto obj_of = [&](int k) -> ObjectPtr {
    return k == 0 ? src : (k >= 1 && k <= (int)refs.size() ? refs[k - 1] : nullptr);
  };
  auto strcol = [&](const ColRef& r) -> const StrCol* {
    ObjectPtr o = obj_of(r.obj);
    if (!o || !o->is_string(r.col)) return nullptr;
    auto it = o->strs.find(r.col);
    return it == o->strs.end() ? nullptr : &it->second;
  };
  auto rewrite = [&](std::string* text, bool allow_bare, const char* what) -> svm_status {
    Expr e;
    std::string err;
    if (!parse_expr(*text, &e, &err)) return SVM_OK;  // the planner reports it
    if (allow_bare && e.nodes[e.root].kind == N_COL && strcol(e.nodes[e.root].ref)) return SVM_OK;
    bool has = false;
    for (const Node& n : e.nodes) has |= n.kind == N_STRCMP || (n.kind == N_COL && strcol(n.ref));
    if (!has) return SVM_OK;
    if (!rewrite_strings(&e, strcol, &err))
      return x->fail(SVM_E_UNSUPPORTED, std::string(what) + " '" + *text + "': " + err);
    *text = print_expr(e, e.root);
    return SVM_OK;
  };
  svm_status st;
  for (auto& f : b->filter_exp)
    if ((st = rewrite(&f, false, "predication"))) return st;
  for (auto& m : b->metric_exp)
    if ((st = rewrite(&m, false, "metric"))) return st;
  for (auto& sel : b->select_exp)
    if ((st = rewrite(&sel, true, "select"))) return st;
  for (size_t j = 0; j < b->join_lkey.size(); j++)
    if (strcol(b->join_lkey[j]) || strcol(b->join_rkey[j]))
      return x->fail(SVM_E_UNSUPPORTED, "String join keys are not supported (join on an int32 key)");
  b->key_hash.assign(b->reduce_key.size(), {});
  for (size_t q = 0; q < b->reduce_key.size(); q++) {
    const ColRef r = b->reduce_key[q];
    if (!strcol(r)) continue;
    ObjectPtr o = obj_of(r.obj);
    int idx;
    if ((st = ensure_rank_col(x, o, r.col, &idx))) return st;
    b->key_hash[q] = o->strs.at(r.col).rank_hash;
    b->reduce_key[q].col = idx;
  }
  return SVM_OK;
}

// Binds a pipeline and resolves its pre_pipeline_id objects.
// Binds `p` (unless `bound`: *b already holds its binding) and finds its
// source and joined objects.
svm_status resolve(Ctx* x, const svm_pipeline* p, Bound* b, ObjectPtr* src, std::vector<ObjectPtr>* refs,
                   bool bound = false) {
  svm_status st = bound ? SVM_OK : bind(x, p, b);
  if (st) return st;
  if (p->npre < 1 || !p->pre_pipeline_id || !p->pre_pipeline_id[0])
    return x->fail(SVM_E_INVALID_ARG, "pipeline " + b->id + " has no source object (pre_pipeline_id[0])");
  // service/service.cu:36-49: every pre_pipeline_id must name a cached object.
  *src = x->find(p->pre_pipeline_id[0]);
  if (!*src) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + p->pre_pipeline_id[0]);
  refs->clear();
  for (int i = 1; i < p->npre; i++) {
    ObjectPtr o = p->pre_pipeline_id[i] ? x->find(p->pre_pipeline_id[i]) : nullptr;
    if (!o)
      return x->fail(SVM_E_NOT_FOUND,
                     std::string("no object ") + (p->pre_pipeline_id[i] ? p->pre_pipeline_id[i] : "(null)"));
    if (o->host)
      return x->fail(SVM_E_UNSUPPORTED, std::string("joined object ") + p->pre_pipeline_id[i] +
                                            " lives in host memory (svm_object_put_host): only a reduce "
                                            "pipeline's fact table may");
    refs->push_back(o);
  }
  if ((*src)->host && !b->is_reduce)
    return x->fail(SVM_E_UNSUPPORTED, std::string("object ") + p->pre_pipeline_id[0] +
                                          " lives in host memory (svm_object_put_host): only a reduce "
                                          "pipeline scans such an object");
  return resolve_strings(x, b, *src, *refs);
}

struct BatchItem {
  std::string id;
  StarPlan plan;
  ObjectPtr src;
  Bound b;
  std::vector<ObjectPtr> refs;
};

// Cost model of a fold, in picoseconds, measured on GB300 with the 256-query
// star-schema mix over a 600 M-row table: one query alone costs about 3.5 ps
// per row it reads (the compiled scans: 90 ms of kernels for the mix's 25.5 G
// query-rows) plus ~90 us of launch, finalize and result handling; the
// batched launch costs about 46 ps per row of the union of the queries'
// ranges (the shared scan, merged-table lookups, bitmaps and per-tile
// bookkeeping: 27.6 ms for the 600 M-row union with the query work removed)
// plus 0.25 ps per query row (6.4 ms for the mix's 25.5 G query-rows), plus
// ~100 us.  The cheaper way runs.
bool batch_is_cheaper(const std::vector<BatchItem>& items) {
  std::vector<std::pair<long long, long long>> iv;
  double single = 0, rows = 0;
  for (const BatchItem& it : items) {
    const long long b = it.plan.P.row_begin, e = it.plan.empty_filter ? b : it.plan.P.row_end;
    iv.push_back({b, e});
    rows += (double)(e - b);
    single += 3.5 * (double)(e - b) + 90e6;
  }
  std::sort(iv.begin(), iv.end());
  double uni = 0;
  long long cb = LLONG_MIN, ce = LLONG_MIN;
  for (auto& v : iv) {
    if (v.first > ce) {
      if (ce > cb) uni += (double)(ce - cb);
      cb = v.first;
      ce = v.second;
    } else {
      ce = std::max(ce, v.second);
    }
  }
  if (ce > cb) uni += (double)(ce - cb);
  const double batch = 46.0 * uni + 0.25 * rows + 100e6;
  return batch < single;
}

// Merged probe tables for a batch: the dense tables probed through each fact
// column, at most 32 per group.  Word 0 of a merged entry holds the group's
// present bits from bit 0 up; payloads (entry >> 1) go first-fit, widest
// first, into the top of word 0 and then into words 1..7.  At most
// kMaxMergedWords words per row and kMaxMergedTables table slots per batch.
//
// Tables of a column whose payload is one bit-packed field share one field
// of the group, wide enough for all their values: the same dimension column
// filtered differently per query (25 part tables, one per category, carry
// the same brand) then costs one field instead of one each.  At a key that
// several of them hold, their values must agree; the merged-table build
// reports any that does not, and such a table keeps a field of its own.
struct MergePlan {
  struct Place {
    int group = -1, slot = -1, present_bit = 0, pay_word = 0, pay_bit = 0;
    bool shared = false;  // the payload sits in the group's shared field
  };
  struct Share {
    int word = 0, bit = 0, bits = 0;  // bits 0: the group has no shared field
    int32_t base = 0;                 // field = value - base
    bool relative = false;            // field = value - the table's own payload minimum (base unused)
  };
  std::map<std::pair<int, const DimTable*>, Place> place;  // (union column, table) -> placement
  std::vector<ProbeGroup> groups;
  std::vector<Share> share;
  std::vector<std::vector<std::pair<DimTablePtr, Place>>> members;
  int nmwords = 0;
  std::vector<int> gtab0;                  // group g owns table slots [gtab0[g], gtab0[g + 1])
};

void plan_merge(Ctx* x, const std::vector<BatchQuery>& qs, const std::vector<BatchItem>& items, MergePlan* mp) {
  std::vector<int> col_order;
  std::map<int, std::vector<DimTablePtr>> by_col;
  for (size_t i = 0; i < qs.size(); i++)
    for (int k = 0; k < qs[i].nsteps; k++) {
      const Step& st = qs[i].steps[k];
      if (st.kind != STEP_PROBE) continue;
      const DimTablePtr& T = items[i].plan.dim_tables[st.dim];
      if (T->desc.layout != LAYOUT_DENSE) continue;
      auto& v = by_col[st.col];
      if (v.empty()) col_order.push_back(st.col);
      if (std::find(v.begin(), v.end(), T) == v.end()) v.push_back(T);
    }
  for (int col : col_order) {
    std::vector<DimTablePtr> tabs = by_col[col];
    std::stable_sort(tabs.begin(), tabs.end(), [](const DimTablePtr& a, const DimTablePtr& z) {
      return a->desc.entry_bits > z->desc.entry_bits;
    });
    auto sharable = [&](const DimTablePtr& T) {
      const DimDesc& d = T->desc;
      return d.npay == 1 && d.pay[0].col == nullptr && d.pay[0].bits > 0 && T->live > 0 && !x->share_refused(T);
    };
    long long smin = LLONG_MAX, smax = LLONG_MIN;
    int nshare = 0, own_bits = 0, rbits = 0;
    for (const DimTablePtr& T : tabs)
      if (sharable(T)) {
        nshare++;
        own_bits += T->desc.pay[0].bits;
        rbits = std::max(rbits, (int)T->desc.pay[0].bits);
        smin = std::min<long long>(smin, T->pay_min[0]);
        smax = std::max<long long>(smax, T->pay_max[0]);
      }
    // The shared field holds value - the tables' common minimum (absolute),
    // or, when narrower, value - each table's own minimum (relative: as wide
    // as the widest table's own range; a key two tables hold must then have
    // the same relative value in both, which the build checks like the
    // absolute field's agreement).
    const int abits = nshare >= 2 ? ceil_log2((unsigned long long)(smax - smin + 1)) : 0;
    const bool relative = nshare >= 2 && rbits < abits;
    const int sbits = relative ? rbits : abits;
    const bool share = nshare >= 2 && sbits < own_bits && sbits <= 31;
    size_t next = 0;
    while (next < tabs.size() && (int)mp->groups.size() < kMaxProbeGroups) {
      // A group takes the column's next tables while their present bits,
      // payloads (8 words) and key span fit; its present region is reserved first.
      const int reserve = (int)std::min<size_t>(32, tabs.size() - next);
      const int g = (int)mp->groups.size();
      mp->groups.push_back(ProbeGroup{col, 1, 0, 0, 0, nullptr});
      mp->share.emplace_back();
      mp->members.emplace_back();
      int ntab = 0, low0 = 32;
      std::vector<int> freebits;  // words 1..
      long long kmin = LLONG_MAX, kmax = LLONG_MIN;
      while (next < tabs.size() && ntab < reserve) {
        const DimTablePtr& T = tabs[next];
        // The payload's used width: fields sit from bit 1 up to the highest
        // field's end (the entry's padding up to entry_bits is not carried).
        int pb = 0;
        for (int f = 0; f < T->desc.npay; f++)
          pb = std::max(pb, (int)T->desc.pay[f].shift + (int)T->desc.pay[f].bits - 1);
        MergePlan::Share& sh = mp->share[g];
        const bool shared = share && sharable(T);
        if (shared) pb = sh.bits ? 0 : sbits;  // the group's shared field, placed by its first table
        const long long tmin = T->desc.key_min, tmax = (long long)T->desc.key_min + T->desc.span - 1;
        const long long nmin = std::min(kmin, tmin), nmax = std::max(kmax, tmax);
        if ((nmax - nmin + 1) * 32ll > (1ll << 30)) break;
        MergePlan::Place pl;
        pl.group = g;
        pl.present_bit = ntab;
        int word = -1;
        if (pb > 0) {
          if (low0 - reserve >= pb) {
            word = 0;
          } else {
            for (size_t z = 0; z < freebits.size() && word < 0; z++)
              if (freebits[z] >= pb) word = (int)z + 1;
            if (word < 0 && freebits.size() < 7) {
              freebits.push_back(32);
              word = (int)freebits.size();
            }
            if (word < 0) break;
          }
          pl.pay_word = word;
          if (word == 0) {
            pl.pay_bit = low0 - pb;
            low0 -= pb;
          } else {
            pl.pay_bit = 32 - freebits[word - 1];
            freebits[word - 1] -= pb;
          }
          if (shared) sh = MergePlan::Share{word, pl.pay_bit, sbits, relative ? 0 : (int32_t)smin, relative};
        }
        if (shared) {
          pl.shared = true;
          pl.pay_word = sh.word;
          pl.pay_bit = sh.bit;
        }
        ntab++;
        next++;
        kmin = nmin;
        kmax = nmax;
        mp->members[g].push_back({T, pl});
        mp->place[{col, T.get()}] = pl;
      }
      if (ntab == 0) {  // the next table alone does not fit: leave it unplaced
        mp->groups.pop_back();
        mp->share.pop_back();
        mp->members.pop_back();
        next++;
        continue;
      }
      ProbeGroup& G = mp->groups[g];
      G.key_min = (int32_t)kmin;
      G.span = (uint32_t)(kmax - kmin + 1);
      G.words = 1 + (int)freebits.size();
    }
  }
  // Groups beyond the per-row word or table-slot budget are left out (their
  // tables unplaced); the others get their words and table slots in order
  // (slot = group's first slot + present bit).
  int off = 0, slots = 0;
  mp->gtab0.assign(mp->groups.size() + 1, 0);
  for (size_t g = 0; g < mp->groups.size(); g++) {
    mp->gtab0[g] = slots;
    if (off + mp->groups[g].words > kMaxMergedWords || slots + (int)mp->members[g].size() > kMaxMergedTables) {
      for (auto& m : mp->members[g]) mp->place.erase({mp->groups[g].col, m.first.get()});
      mp->members[g].clear();
      mp->groups[g].words = 0;
      continue;
    }
    mp->groups[g].word_off = off;
    for (auto& m : mp->members[g]) {
      m.second.slot = slots + m.second.present_bit;
      mp->place[{mp->groups[g].col, m.first.get()}].slot = m.second.slot;
    }
    slots += (int)mp->members[g].size();
    off += mp->groups[g].words;
  }
  mp->gtab0[mp->groups.size()] = slots;
  mp->nmwords = off;
}

// The merged table of group g, from the cache or built now.  A table built
// now with a shared field reports its sources' disagreements into
// `*conflict` (device) and its cache key into `*checked`.
svm_status merged_table(Ctx* x, MergePlan* mp, int g, unsigned int* conflict, std::string* checked) {
  ProbeGroup& G = mp->groups[g];
  const MergePlan::Share& sh = mp->share[g];
  std::string key = std::to_string(G.key_min) + ":" + std::to_string(G.span) + ":" + std::to_string(G.words);
  for (auto& m : mp->members[g]) {
    key += "|" + std::to_string((uintptr_t)m.first.get()) + "@" + std::to_string(m.second.present_bit) + "." +
           std::to_string(m.second.pay_word) + "." + std::to_string(m.second.pay_bit);
    if (m.second.shared) key += "s" + std::to_string(sh.bits) + "." + std::to_string(sh.base) + (sh.relative ? "r" : "");
  }
  checked->clear();
  auto it = x->merged_cache.find(key);
  if (it == x->merged_cache.end()) {
    if (x->merged_cache.size() >= 64) {  // evict the least recently used
      auto old = x->merged_cache.begin();
      for (auto c = x->merged_cache.begin(); c != x->merged_cache.end(); ++c)
        if (c->second.stamp < old->second.stamp) old = c;
      x->merged_cache.erase(old);
    }
    MergedTable mt;
    svm_status st = x->alloc((size_t)G.span * G.words * 4, &mt.buf);
    if (st) return st;
    for (size_t b0 = 0; b0 < mp->members[g].size(); b0 += kMaxMergeSrcs) {
      // More members than one build holds: OR further builds in (all start from zero).
      MergeBuild mb{};
      mb.key_min = G.key_min;
      mb.span = G.span;
      mb.words = G.words;
      mb.conflict = conflict;
      for (size_t i = b0; i < mp->members[g].size() && mb.nsrc < kMaxMergeSrcs; i++) {
        const auto& m = mp->members[g][i];
        const DimDesc& d = m.first->desc;
        int pb = 0;
        for (int f = 0; f < d.npay; f++) pb = std::max(pb, (int)d.pay[f].shift + (int)d.pay[f].bits - 1);
        const int32_t off =
            m.second.shared && !sh.relative ? (int32_t)((uint32_t)d.pay[0].min - (uint32_t)sh.base) : 0;
        mb.src[mb.nsrc++] = MergeSrc{d.words,          d.key_min,          d.span, d.entry_bits,
                                     m.second.present_bit, m.second.pay_word, m.second.pay_bit, pb,
                                     m.second.shared ? 1 : 0, off};
        if (m.second.shared) *checked = key;
        mt.srcs.push_back(m.first);
      }
      if (b0 > 0) return x->fail(SVM_E_UNSUPPORTED, "more than 32 tables in one merged probe group");
      cudaError_t e = launch_merge_build(mb, (uint32_t*)mt.buf->p, x->stream);
      if (e) return x->cuda_fail(e, "merged table build");
    }
    it = x->merged_cache.emplace(key, std::move(mt)).first;
  }
  it->second.stamp = ++x->merged_stamp;
  G.table = (const uint32_t*)it->second.buf->p;
  return SVM_OK;
}

// One batched launch over queries that share a fact table: queries whose
// probes all hit merged tables run in the merged kernel, the others in the
// per-query batch kernel; one finalize covers both.
// A batch enqueued without waiting (svm_batch_begin): its device buffers,
// the result store sized for every group the queries can produce, and the
// slots in the fold's pinned host buffer where its result bounds and error
// word arrive.  Completed by finish_part once the fold's event has fired.
struct FoldPart {
  std::vector<BatchItem> items;
  std::vector<int> order;            // launch order -> items index
  DevBufPtr dev;                     // descriptors, slots, finalize scratch, bounds, error word
  ObjectPtr store;                   // 3 int32 key columns + 3 int64 sum columns
  size_t host_off = 0;               // first uint64 of this part in the fold's pinned buffer
  int nq = 0;
};

// A fold in flight: every pipeline of an svm_batch_begin call, in input
// order.  A reduce pipeline batched into part `part` at launch position
// `pos` is completed when the fold's event fires; every other pipeline (a
// Map, one the batch kernel does not take, one run alone by the cost model)
// ran to completion inside svm_batch_begin.  With host results requested,
// each part's whole result store and each completed pipeline's columns are
// copied behind the fold's work into pinned staging.
struct Fold {
  struct Res {
    std::string id;
    int part = -1, pos = -1;
    ObjectPtr done;                  // completed inside begin
    size_t stage_off = 0;            // completed: its columns' first byte in staging
  };
  std::vector<Res> res;
  std::vector<FoldPart> parts;
  std::vector<size_t> part_stage;    // per part: first byte of its store copy in staging
  std::vector<unsigned long long> part_groups;  // per part: store rows
  bool want_host = false;
  PinnedBlock bounds, stage;         // pinned: per part nq + 2 words; the result copies
  cudaEvent_t done = nullptr;
};

// Each batched query's result object: a view of its rows [hb[j], hb[j + 1])
// in the batch's result store (j its launch position).
svm_status store_batch_results(Ctx* x, const std::vector<BatchItem>& items, const std::vector<int>& order,
                               const ObjectPtr& all, const unsigned long long* hb) {
  for (size_t j = 0; j < order.size(); j++) {
    const BatchItem& it = items[order[j]];
    auto out = std::make_shared<Object>();
    out->id = it.id;
    out->version = x->next_version++;
    out->ncols = it.plan.nkeys + it.plan.nmet;
    out->types = it.plan.out_types;
    for (int k = 0; k < it.plan.nkeys; k++) out->storage.push_back(all->storage[k]);
    for (int m = 0; m < it.plan.nmet; m++) out->storage.push_back(all->storage[kMaxKeys + m]);
    out->row0 = hb[j];
    out->nrows = hb[j + 1] - out->row0;
    out->has_bulks = true;
    out->bulk0_rows = out->nrows;
    out->source_rows = out->nrows;
    svm_status st = translate_keys(x, it.b, out);
    if (st) return st;
    x->put_object(it.id, out);
  }
  return SVM_OK;
}

svm_status exec_batch(Ctx* x, std::vector<BatchItem>& items, FoldPart* async_part = nullptr,
                      unsigned long long* host_bounds = nullptr) {
  const int nq = (int)items.size();
  // Union of the fact columns, identified by their storage.
  std::vector<const void*> ucols;
  auto uslot = [&](const void* base) {
    for (size_t i = 0; i < ucols.size(); i++)
      if (ucols[i] == base) return (int)i;
    ucols.push_back(base);
    return (int)ucols.size() - 1;
  };
  std::vector<BatchQuery> qs(nq);
  for (int i = 0; i < nq; i++) {
    StarPlan& pl = items[i].plan;
    StarParams& P = pl.P;
    BatchQuery& Q = qs[i];
    std::vector<int> remap(pl.fact_cols.size());
    for (size_t c = 0; c < pl.fact_cols.size(); c++) remap[c] = uslot(items[i].src->base(pl.fact_cols[c]));
    Q.row_begin = P.row_begin;
    Q.row_end = pl.empty_filter ? P.row_begin : P.row_end;
    Q.nsteps = P.nsteps;
    for (int k = 0; k < P.nsteps; k++) {
      Q.steps[k] = P.steps[k];
      Q.steps[k].col = remap[P.steps[k].col];
      Q.steps[k].smem_word_off = -1;  // batch mode probes every table in global memory
    }
    auto fix = [&](Extract e) {
      if (e.dim < 0) e.slot = remap[e.slot];
      return e;
    };
    Q.nkeys = P.nkeys;
    for (int k = 0; k < P.nkeys; k++) {
      Q.kx[k] = fix(P.kx[k]);
      Q.kmin[k] = P.kmin[k];
      Q.krange[k] = P.krange[k];
      Q.kstride[k] = (uint32_t)P.kstride[k];
    }
    Q.nmetrics = P.nmetrics;
    for (int m = 0; m < P.nmetrics; m++) {
      Q.mform[m] = P.metrics[m].form;
      Q.xa[m] = fix(P.metrics[m].xa);
      Q.xb[m] = fix(P.metrics[m].xb);
    }
    Q.ngroups = P.ngroups;
  }
  if ((int)ucols.size() > kMaxBatchCols) return x->fail(SVM_E_UNSUPPORTED, "batch reads more than 12 fact columns");

  // ---- merged probe groups, and the queries they cover
  MergePlan mp;
  std::vector<int> order;
  std::vector<MQuery> mqs;
  std::vector<const int32_t*> gcols;
  int nmerged = 0;
  svm_status st;
  // Shared memory of the merged kernel without descriptors (two-stage ring);
  // each query adds its resident descriptor.
  const size_t kMergedSmem = 226 * 1024, kPerQuery = sizeof(MQuery) + 8 + 8 + 4 + 4;
  auto merged_fixed = [&](int nst) {
    BatchParams T{};
    T.ncols = (int)ucols.size();
    T.nstages = nst;
    T.nmwords = mp.nmwords;
    return mbatch_smem_bytes(T);
  };
  for (;;) {
    mp = MergePlan{};
    order.clear();
    gcols.clear();
    mqs.assign(nq, MQuery{});
    plan_merge(x, qs, items, &mp);
    if (merged_fixed(2) + kPerQuery > kMergedSmem) mp.place.clear();  // every query takes the per-query kernel
    std::vector<int> legacy;
    for (int i = 0; i < nq; i++) {
      BatchQuery& Q = qs[i];
      struct DimPlace {
        bool ok = false;
        MergePlan::Place p;
      } dp[kMaxDims];
      bool ok = true;
      for (int k = 0; k < Q.nsteps && ok; k++) {
        const Step& st = Q.steps[k];
        if (st.kind != STEP_PROBE) continue;
        auto f = mp.place.find({st.col, items[i].plan.dim_tables[st.dim].get()});
        if (f == mp.place.end() || mp.groups[f->second.group].words == 0) {
          ok = false;
          break;
        }
        dp[st.dim].ok = true;
        dp[st.dim].p = f->second;
      }
      if (!ok) {
        legacy.push_back(i);
        continue;
      }
      order.push_back(i);
      // The merged kernel's descriptor: probe steps become table-slot bit tests
      // (a folded key range becomes a range step), then the range steps.
      MQuery M{};
      M.row_begin = Q.row_begin;
      M.row_end = Q.row_end;
      M.ngroups = (uint32_t)Q.ngroups;
      bool fits = true;
      for (int k = 0; k < Q.nsteps; k++) {
        const Step& st = Q.steps[k];
        if (st.kind == STEP_PROBE) {
          const MergePlan::Place& pl = dp[st.dim].p;
          M.probe_tab[M.nprobe++] = (uint8_t)pl.slot;
          M.gmask |= 1u << pl.group;
          if (st.lo == INT_MIN && st.hi == INT_MAX) continue;
        }
        if (M.nrange == kMaxMRanges) {
          fits = false;
          break;
        }
        M.range_col[M.nrange] = (uint8_t)st.col;
        M.range_lo[M.nrange] = st.lo;
        M.range_hi[M.nrange] = st.hi;
        M.nrange++;
      }
      auto mxt = [&](const Extract& e) {
        MExtract r{};
        r.mask = e.mask;
        r.base = e.base;
        if (e.dim < 0) {
          r.src = -1;
          r.slot = (uint8_t)e.slot;
          return r;
        }
        // A payload field at bit `shift` of the entry sits at pay_bit + shift - 1
        // of the payload word (the present bit is not carried there).
        const MergePlan::Place& pl = dp[e.dim].p;
        r.src = (int8_t)mp.groups[pl.group].word_off;
        r.slot = (uint8_t)pl.pay_word;
        r.sg = (uint8_t)mp.groups[pl.group].words;
        r.shift = (uint8_t)(pl.pay_bit + (e.mask ? e.shift - 1 : 0));
        if (pl.shared && e.mask) {  // the group's shared field holds value - sh.base (or - the table's minimum)
          const MergePlan::Share& sh = mp.share[pl.group];
          const DimDesc& d = items[i].plan.dim_tables[e.dim]->desc;
          r.shift = (uint8_t)sh.bit;
          r.mask = sh.bits >= 32 ? 0xFFFFFFFFu : (1u << sh.bits) - 1u;
          if (!sh.relative) r.base = (int32_t)((uint32_t)e.base - (uint32_t)d.pay[0].min + (uint32_t)sh.base);
        }
        if (e.col) {
          size_t gi = std::find(gcols.begin(), gcols.end(), e.col) - gcols.begin();
          if (gi == gcols.size()) {
            if (gcols.size() == (size_t)kMaxGatherCols) {
              fits = false;
              return r;
            }
            gcols.push_back(e.col);
          }
          r.sg |= (uint8_t)((gi + 1) << 4);
        }
        M.gmask |= 1u << pl.group;
        return r;
      };
      M.nkeys = (uint8_t)Q.nkeys;
      for (int k = 0; k < Q.nkeys; k++) {
        M.kx[k] = mxt(Q.kx[k]);
        M.krange[k] = Q.krange[k];
        M.kstride[k] = Q.kstride[k];
      }
      M.nmetrics = (uint8_t)Q.nmetrics;
      for (int m = 0; m < Q.nmetrics; m++) {
        M.mform[m] = (uint8_t)Q.mform[m];
        M.xa[m] = mxt(Q.xa[m]);
        if (Q.mform[m] != MF_OPND) M.xb[m] = mxt(Q.xb[m]);
      }
      if (!fits) {  // more range steps or gather columns than the descriptor holds
        order.pop_back();
        legacy.push_back(i);
        continue;
      }
      mqs[i] = M;
    }
    nmerged = (int)order.size();
    // Consumer warps claim a tile's queries in descriptor order and wait for
    // the last at the tile's end: the most aggregation work first (longest
    // processing time first) keeps that tail short.
    std::stable_sort(order.begin(), order.end(), [&](int a, int z) {
      const StarPlan& pa = items[a].plan;
      const StarPlan& pz = items[z].plan;
      return pa.est_pass * (pa.nkeys + pa.nmet + 1) > pz.est_pass * (pz.nkeys + pz.nmet + 1);
    });
    order.insert(order.end(), legacy.begin(), legacy.end());
    if (!nmerged) break;
    // Build the merged tables; a shared field that two of its tables
    // disagree on sends those tables to fields of their own, and the batch
    // is planned again (each round refuses at least one more table).
    DevBufPtr conflict;
    if ((st = x->alloc(4 * mp.groups.size(), &conflict, true))) return st;
    std::vector<std::string> checked(mp.groups.size());
    auto unchecked = [&](svm_status r) {  // no table leaves unchecked in the cache
      for (const std::string& k : checked)
        if (!k.empty()) x->merged_cache.erase(k);
      return r;
    };
    bool any_checked = false;
    for (size_t g = 0; g < mp.groups.size(); g++) {
      if (!mp.groups[g].words) continue;
      if ((st = merged_table(x, &mp, (int)g, (unsigned int*)conflict->p + g, &checked[g]))) return unchecked(st);
      any_checked |= !checked[g].empty();
    }
    if (!any_checked) break;
    std::vector<unsigned int> bad(mp.groups.size());
    cudaError_t ce = cudaMemcpyAsync(bad.data(), conflict->p, 4 * bad.size(), cudaMemcpyDeviceToHost, x->stream);
    if (!ce) ce = cudaStreamSynchronize(x->stream);
    if (ce) return unchecked(x->cuda_fail(ce, "merged table check"));
    bool refused = false;
    for (size_t g = 0; g < mp.groups.size(); g++) {
      if (!bad[g]) continue;
      for (size_t i = 0; i < mp.members[g].size(); i++)
        if (bad[g] >> i & 1u) x->no_share[mp.members[g][i].first.get()] = mp.members[g][i].first;
      x->merged_cache.erase(checked[g]);
      refused = true;
    }
    if (!refused) break;
  }

  // ---- slots and group numbering in launch order
  std::vector<BatchQuery> dqs(nq);
  std::vector<MQuery> dmq(nmerged);
  unsigned long long slot_words = 0, total_groups = 0;
  long long lo[2] = {LLONG_MAX, LLONG_MAX}, hi[2] = {LLONG_MIN, LLONG_MIN};
  for (int j = 0; j < nq; j++) {
    BatchQuery Q = qs[order[j]];
    Q.slot_off = slot_words;
    Q.group_off = total_groups;
    slot_words += (unsigned long long)(Q.nmetrics + 1) * Q.ngroups;
    total_groups += Q.ngroups;
    const int part = j < nmerged ? 0 : 1;
    lo[part] = std::min(lo[part], Q.row_begin);
    hi[part] = std::max(hi[part], Q.row_end);
    dqs[j] = Q;
    if (part == 0) {
      mqs[order[j]].slot_off = Q.slot_off;
      dmq[j] = mqs[order[j]];
    }
  }
  const size_t qbytes = sizeof(BatchQuery) * nq, mbytes = sizeof(MQuery) * nmerged;
  const size_t fin_words = (total_groups + 1) / 2 + 1 + total_groups + 1 + scan_tmp_words(total_groups);
  // Merged launches: as many queries per launch as their descriptors fit.
  int mst = 2;
  for (int nst = kStages; nst > 2; nst--)
    if (merged_fixed(nst) + kPerQuery * nmerged <= kMergedSmem) {
      mst = nst;
      break;
    }
  const int per_launch = nmerged ? (int)((kMergedSmem - merged_fixed(mst)) / kPerQuery) : 1;
  const int nlaunch = nmerged ? (nmerged + per_launch - 1) / per_launch : 0;
  const size_t need = qbytes + mbytes + 8 * slot_words + 8 * (nlaunch + 1) + 8 * fin_words + 8 * (nq + 2) + 8 * 1024;
  void *dq, *dm = nullptr, *slots, *ctr, *fin, *bounds;
  int* err_word = x->d_error;
  if (async_part) {
    // The fold's own device buffer (carved like the scratch arena), so that
    // folds in flight never share scratch.
    if ((st = x->alloc(need, &async_part->dev))) return st;
    char* base = (char*)async_part->dev->p;
    size_t used = 0;
    auto take = [&](size_t bytes) {
      void* p = base + used;
      used += (bytes + 255) & ~size_t(255);
      return p;
    };
    dq = take(qbytes);
    if (nmerged) dm = take(mbytes);
    slots = take(8 * slot_words);
    ctr = take(8 * (nlaunch + 1));
    fin = take(8 * fin_words);
    bounds = take(8 * (nq + 2));
    err_word = (int*)((unsigned long long*)bounds + nq + 1);
  } else {
    x->scratch_reset();
    if ((st = x->scratch_reserve(need))) return st;
    if ((st = x->scratch_take(qbytes, &dq)) || (nmerged && (st = x->scratch_take(mbytes, &dm))) ||
        (st = x->scratch_take(8 * slot_words, &slots)) || (st = x->scratch_take(8 * (nlaunch + 1), &ctr)) ||
        (st = x->scratch_take(8 * fin_words, &fin)) || (st = x->scratch_take(8 * (nq + 1), &bounds)))
      return st;
  }
  cudaError_t e = cudaMemcpyAsync(dq, dqs.data(), qbytes, cudaMemcpyHostToDevice, x->stream);
  if (!e && async_part) e = cudaMemsetAsync(err_word, 0, 8, x->stream);
  if (!e && nmerged) e = cudaMemcpyAsync(dm, dmq.data(), mbytes, cudaMemcpyHostToDevice, x->stream);
  if (!e) e = cudaMemsetAsync(slots, 0, 8 * slot_words, x->stream);
  if (!e) e = cudaMemsetAsync(ctr, 0, 8 * (nlaunch + 1), x->stream);
  if (e) return x->cuda_fail(e, "batch setup");
  cudaEvent_t ev;
  for (int part = 0; part <= nlaunch; part++) {
    const bool merged = part < nlaunch;
    const int q0 = merged ? part * per_launch : nmerged;
    const int qn = merged ? std::min(per_launch, nmerged - q0) : nq - nmerged;
    if (!qn) continue;
    BatchParams B{};
    B.ncols = (int)ucols.size();
    for (size_t c = 0; c < ucols.size(); c++) B.cols[c] = (const int32_t*)ucols[c];
    long long rb = LLONG_MAX, re = LLONG_MIN;
    for (int j = q0; j < q0 + qn; j++) {
      rb = std::min(rb, dqs[j].row_begin);
      re = std::max(re, dqs[j].row_end);
    }
    B.row_begin = rb;
    B.row_end = std::max(re, rb);
    B.queries = (const BatchQuery*)dq + q0;
    B.nqueries = qn;
    B.slots = (unsigned long long*)slots;
    B.tile_counter = (unsigned long long*)ctr + part;
    B.error = err_word;
    if (merged) {
      B.nprobe = (int)mp.groups.size();
      for (size_t g = 0; g < mp.groups.size(); g++) B.probe[g] = mp.groups[g];
      B.nmwords = mp.nmwords;
      B.mq = (const MQuery*)dm + q0;
      for (size_t g = 0; g < mp.gtab0.size(); g++) B.gtab0[g] = mp.gtab0[g];
      for (size_t c = 0; c < gcols.size(); c++) B.gcol[c] = gcols[c];
      B.nstages = mst;
      B.cwarps = kMBatchWarps;
      // Launch configuration of the merged kernel: the consumer / fill warp
      // split (28 + 4 or 24 + 8) and the ring depth (at most the rule's,
      // which fits every descriptor of the launch).  The rule: 28 + 4, the
      // deepest ring.  With autotuning, the first launch of a batch shape
      // times every candidate on the batch itself (this launch's slots and
      // tile counter zeroed before each and again after -- only this
      // launch's: the fold's earlier launches have already written theirs),
      // and the fastest is kept.  A fold begun without waiting never times
      // candidates (that would wait for the device inside svm_batch_begin and
      // hold up the folds behind it): it takes the choice cached for its
      // batch shape, else the rule.
      std::vector<std::pair<int, int>> cands;  // (consumer warps, ring stages)
      for (int cw : {28, 24})
        for (int nst = mst; nst >= 2; nst--)
          if ((!x->pin_batch_cw || cw == x->pin_batch_cw) && (!x->pin_batch_stages || nst == x->pin_batch_stages))
            cands.push_back({cw, nst});
      if (cands.empty()) return x->fail(SVM_E_UNSUPPORTED, "no batch launch configuration fits the pinned choices");
      std::pair<int, int> pick = cands[0];
      bool tuned = false;
      const std::string key = "q" + std::to_string(ceil_log2((unsigned long long)qn + 1)) + ":c" +
                              std::to_string(B.ncols) + ":w" + std::to_string(B.nmwords) + ":g" +
                              std::to_string(B.nprobe) + ":s" + std::to_string(mst) + ":pin" +
                              std::to_string(x->pin_batch_cw) + "," + std::to_string(x->pin_batch_stages);
      if (x->cfg.autotune && cands.size() > 1) {
        auto hit = x->batch_tune.find(key);
        if (hit != x->batch_tune.end()) {
          pick = hit->second;
          tuned = true;
        } else if (!async_part) {
          // This launch's queries own one contiguous run of slots.
          const BatchQuery& ql = dqs[q0 + qn - 1];
          const unsigned long long s_lo = dqs[q0].slot_off;
          const unsigned long long s_hi = ql.slot_off + (unsigned long long)(ql.nmetrics + 1) * ql.ngroups;
          unsigned long long* part_slots = (unsigned long long*)slots + s_lo;
          const size_t part_bytes = 8 * (size_t)(s_hi - s_lo);
          cudaEvent_t t0, t1;
          cudaEventCreate(&t0);
          cudaEventCreate(&t1);
          float best = 0.f;
          for (const auto& c : cands) {
            B.cwarps = c.first;
            B.nstages = c.second;
            const size_t sm = mbatch_smem_bytes(B);
            const int g = mbatch_grid_size(B, sm);
            if (g <= 0) continue;
            if (!e) e = cudaMemsetAsync(part_slots, 0, part_bytes, x->stream);
            if (!e) e = cudaMemsetAsync(B.tile_counter, 0, 8, x->stream);
            if (!e) e = cudaEventRecord(t0, x->stream);
            if (!e) e = launch_mbatch(B, g, sm, x->stream);
            if (!e) e = cudaEventRecord(t1, x->stream);
            if (!e) e = cudaEventSynchronize(t1);
            float ms = 0.f;
            if (!e) e = cudaEventElapsedTime(&ms, t0, t1);
            if (e) break;
            if (best == 0.f || ms < best) {
              best = ms;
              pick = c;
            }
          }
          cudaEventDestroy(t0);
          cudaEventDestroy(t1);
          if (!e) e = cudaMemsetAsync(part_slots, 0, part_bytes, x->stream);
          if (!e) e = cudaMemsetAsync(B.tile_counter, 0, 8, x->stream);
          if (e) return x->cuda_fail(e, "batch kernel tuning");
          x->batch_tune[key] = pick;
          tuned = true;
        }
      }
      B.cwarps = pick.first;
      B.nstages = pick.second;
      const size_t smem = mbatch_smem_bytes(B);
      const int grid = mbatch_grid_size(B, smem);
      x->last_launch = "{\"kernel\": \"batch\", \"consumer_warps\": " + std::to_string(pick.first) +
                       ", \"fill_warps\": " + std::to_string(32 - pick.first) + ", \"ring_stages\": " +
                       std::to_string(pick.second) + ", \"queries_per_launch\": " + std::to_string(per_launch) +
                       ", \"merged_launches\": " + std::to_string(nlaunch) + ", \"queries\": " +
                       std::to_string(nq) + ", \"grid\": " + std::to_string(grid) + ", \"smem_bytes\": " +
                       std::to_string(smem) + ", \"tuned\": " + (tuned ? "true" : "false") + "}";
      if (grid <= 0) {
        int regs = 0, maxt = 0;
        size_t ss = 0;
        mbatch_attributes(&regs, &maxt, &ss);
        return x->fail(SVM_E_UNSUPPORTED, "merged batch kernel does not fit an SM: " + std::to_string(smem) +
                                              " B dynamic + " + std::to_string(ss) + " B static shared memory, " +
                                              std::to_string(regs) + " registers, max " + std::to_string(maxt) +
                                              " threads per block");
      }
      x->prof_begin(SVM_K_BATCH, &ev);
      e = launch_mbatch(B, grid, smem, x->stream);
      x->prof_end(SVM_K_BATCH, ev);
    } else {
      B.nstages = 2;
      for (int nst = kStages; nst >= 2; nst--) {
        B.nstages = nst;
        if (batch_smem_bytes(B) <= 100 * 1024) break;
      }
      const size_t smem = batch_smem_bytes(B);
      x->prof_begin(SVM_K_BATCH, &ev);
      e = launch_batch(B, batch_grid_size(B, smem), smem, x->stream);
      x->prof_end(SVM_K_BATCH, ev);
    }
    if (e) return x->cuda_fail(e, "batch kernel");
  }
  const BatchQuery* dQ = (const BatchQuery*)dq;
  uint32_t* flags = (uint32_t*)fin;
  unsigned long long* pos = (unsigned long long*)fin + (total_groups + 1) / 2 + 1;
  unsigned long long* scant = pos + total_groups + 1;
  x->prof_begin(SVM_K_FINALIZE, &ev);
  e = launch_batch_finalize(dQ, nq, (unsigned long long*)slots, total_groups, flags, pos, scant, nullptr, x->stream);
  x->prof_end(SVM_K_FINALIZE, ev);
  if (!e) e = launch_batch_bounds(dQ, nq, pos, total_groups, (unsigned long long*)bounds, x->stream);
  if (e) return x->cuda_fail(e, "batch finalize");
  if (async_part) {
    // No host step: the store holds every group the queries can produce, the
    // rows are written now, and the bounds and the error word go to the
    // fold's pinned buffer behind them.
    std::vector<int> types = {SVM_INT32, SVM_INT32, SVM_INT32, SVM_INT64, SVM_INT64, SVM_INT64};
    ObjectPtr all = new_result_object(x, "", types, total_groups, &st);
    if (st) return st;
    BatchOut o{};
    for (int k = 0; k < kMaxKeys; k++) o.key[k] = (int32_t*)all->col(k);
    for (int m = 0; m < kMaxMetrics; m++) o.sum[m] = (long long*)all->col(kMaxKeys + m);
    x->prof_begin(SVM_K_FINALIZE, &ev);
    e = launch_batch_finalize(dQ, nq, (unsigned long long*)slots, total_groups, flags, pos, scant, &o, x->stream);
    x->prof_end(SVM_K_FINALIZE, ev);
    if (!e) e = cudaMemcpyAsync(host_bounds, bounds, 8 * (nq + 2), cudaMemcpyDeviceToHost, x->stream);
    if (e) return x->cuda_fail(e, "batch write");
    async_part->store = all;
    async_part->order = order;
    async_part->nq = nq;
    async_part->items = std::move(items);
    return SVM_OK;
  }
  // Only each query's first result row comes back to the host.
  std::vector<unsigned long long> hb(nq + 1);
  if (!e) e = cudaMemcpyAsync(hb.data(), bounds, 8 * (nq + 1), cudaMemcpyDeviceToHost, x->stream);
  if (e) return x->cuda_fail(e, "batch finalize");
  if ((st = sync_and_check(x, "batch"))) return st;
  // One result store for the batch; each query's rows are a slice of it.
  const unsigned long long rows = hb[nq];
  std::vector<int> types = {SVM_INT32, SVM_INT32, SVM_INT32, SVM_INT64, SVM_INT64, SVM_INT64};
  ObjectPtr all = new_result_object(x, "", types, rows, &st);
  if (st) return st;
  BatchOut o{};
  for (int k = 0; k < kMaxKeys; k++) o.key[k] = (int32_t*)all->col(k);
  for (int m = 0; m < kMaxMetrics; m++) o.sum[m] = (long long*)all->col(kMaxKeys + m);
  x->prof_begin(SVM_K_FINALIZE, &ev);
  e = launch_batch_finalize(dQ, nq, (unsigned long long*)slots, total_groups, flags, pos, scant, &o, x->stream);
  x->prof_end(SVM_K_FINALIZE, ev);
  if (e) return x->cuda_fail(e, "batch write");
  if ((st = sync_and_check(x, "batch write"))) return st;
  return store_batch_results(x, items, order, all, hb.data());
}

}  // namespace

svm_status pipeline_footprint(Ctx* x, const svm_pipeline* p, unsigned long long* bytes) {
  Bound b;
  ObjectPtr src;
  std::vector<ObjectPtr> refs;
  svm_status st = resolve(x, p, &b, &src, &refs);
  if (st) return st;
  if (!b.is_reduce) {  // at most every source row, every output column
    unsigned long long per_row = 0;
    for (const auto& c : b.sink) per_row += c.type == SVM_INT64 ? 8 : 4;
    *bytes = (src->nrows + 64) * per_row + 4096;
    return SVM_OK;
  }
  StarPlan plan;
  if ((st = plan_star_cached(x, b, src, refs, &plan))) return st;
  const unsigned long long G = plan.P.ngroups;
  // group slots + finalize flags/positions + at most G result rows
  *bytes = 8 * (plan.nmet + 1) * G + 16 * (G + 1) + (4ull * plan.nkeys + 8ull * plan.nmet) * G + 4096;
  return SVM_OK;
}

svm_status run_pipeline(Ctx* x, const svm_pipeline* p) {
  Bound b;
  ObjectPtr src;
  std::vector<ObjectPtr> refs;
  svm_status st = resolve(x, p, &b, &src, &refs);
  if (st) return st;
  if (!b.is_reduce) return run_select(x, b, src, refs);
  return run_star(x, b, src, refs);
}

svm_status run_batch(Ctx* x, int n, const svm_pipeline* p) {
  // Select pipelines run first, in order (fact pipelines may join their outputs);
  // reduce pipelines over the same fact table share one batched launch.  A
  // batch in which some pipeline reads a reduce pipeline's output runs in order.
  std::vector<char> reduce(n);
  std::vector<Bound> bounds(n);
  std::set<std::string> reduce_ids;
  for (int i = 0; i < n; i++) {
    svm_status st = bind(x, &p[i], &bounds[i]);
    if (st) return st;
    reduce[i] = bounds[i].is_reduce;
    if (bounds[i].is_reduce) reduce_ids.insert(bounds[i].id);
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < p[i].npre; j++)
      if (p[i].pre_pipeline_id && p[i].pre_pipeline_id[j] && reduce_ids.count(p[i].pre_pipeline_id[j])) {
        for (int k = 0; k < n; k++) {
          svm_status st = run_pipeline(x, &p[k]);
          if (st) return st;
        }
        return SVM_OK;
      }
  for (int i = 0; i < n; i++) {
    svm_status st;
    if (!reduce[i] && (st = run_pipeline(x, &p[i]))) return st;
  }
  std::map<const void*, std::vector<BatchItem>> groups;
  for (int i = 0; i < n; i++) {
    if (!reduce[i]) continue;
    Bound& b = bounds[i];  // bound above (binding parses the pipeline alone, reading no object)
    ObjectPtr src;
    std::vector<ObjectPtr> refs;
    svm_status st = resolve(x, &p[i], &b, &src, &refs, true);
    if (st) return st;
    BatchItem it;
    it.id = b.id;
    it.src = src;
    it.b = b;
    it.refs = refs;
    if ((st = plan_star_cached(x, b, src, refs, &it.plan))) return st;
    bool eligible = !it.plan.empty_src && !it.plan.needs_prog && !src->host;
    for (int m = 0; m < it.plan.nmet; m++) eligible &= it.plan.wide[m] != 0;
    if (!eligible) {
      if ((st = run_star(x, b, src, refs))) return st;
      continue;
    }
    groups[src->storage[0].get()].push_back(std::move(it));
  }
  for (auto& g : groups) {
    // Slot arrays and group numbering stay within 32-bit-friendly bounds per launch.
    std::vector<BatchItem>& items = g.second;
    const int policy = x->cfg.batch_policy;
    if (policy == SVM_BATCH_NEVER || (policy == SVM_BATCH_AUTO && !batch_is_cheaper(items))) {
      for (BatchItem& it : items) {
        svm_status st = run_star(x, it.b, it.src, it.refs);
        if (st) return st;
      }
      continue;
    }
    for (size_t b0 = 0; b0 < items.size(); b0 += 1024) {
      std::vector<BatchItem> part(std::make_move_iterator(items.begin() + b0),
                                  std::make_move_iterator(items.begin() + std::min(items.size(), b0 + 1024)));
      svm_status st = exec_batch(x, part);
      if (st) return st;
    }
  }
  return SVM_OK;
}


// ============================================================ folds in flight
namespace {

// Bytes of a result's host copy in svm_objects_read's layout: every column
// starts 8-byte aligned.
unsigned long long host_bytes(const std::vector<int>& types, unsigned long long rows) {
  unsigned long long b = 0;
  for (int t : types) b += (rows * (t == SVM_INT64 ? 8 : 4) + 7) & ~7ull;
  return b;
}

svm_status fold_fail(Ctx* x, Fold* f, svm_status st) {
  // Nothing of the fold may still be running when its buffers go back.
  cudaStreamSynchronize(x->stream);
  x->pinned_give(&f->bounds);
  x->pinned_give(&f->stage);
  if (f->done) cudaEventDestroy(f->done);
  delete f;
  return st;
}

}  // namespace

svm_status batch_begin(Ctx* x, int n, const svm_pipeline* p, int want_host, void** out) {
  *out = nullptr;
  auto* F = new Fold;
  F->want_host = want_host != 0;
  F->res.resize(n);
  std::vector<Bound> bounds(n);
  std::vector<char> reduce(n);
  std::set<std::string> reduce_ids;
  svm_status st;
  for (int i = 0; i < n; i++) {
    if ((st = bind(x, &p[i], &bounds[i]))) return fold_fail(x, F, st);
    F->res[i].id = bounds[i].id;
    reduce[i] = bounds[i].is_reduce;
    if (reduce[i]) reduce_ids.insert(bounds[i].id);
  }
  if ((st = x->pinned_take(8 * (3 * (size_t)n + 2), &F->bounds))) return fold_fail(x, F, st);
  auto complete_now = [&](int i) -> svm_status {
    svm_status r = run_pipeline(x, &p[i]);
    if (!r) F->res[i].done = x->find(F->res[i].id);
    return r;
  };
  bool dependent = false;  // a pipeline reads another's reduce output: everything in order, now
  for (int i = 0; i < n && !dependent; i++)
    for (int j = 0; j < p[i].npre; j++)
      if (p[i].pre_pipeline_id && p[i].pre_pipeline_id[j] && reduce_ids.count(p[i].pre_pipeline_id[j]))
        dependent = true;
  if (dependent) {
    for (int i = 0; i < n; i++)
      if ((st = complete_now(i))) return fold_fail(x, F, st);
  } else {
    for (int i = 0; i < n; i++)
      if (!reduce[i] && (st = complete_now(i))) return fold_fail(x, F, st);
    std::map<const void*, std::vector<std::pair<int, BatchItem>>> groups;
    for (int i = 0; i < n; i++) {
      if (!reduce[i]) continue;
      ObjectPtr src;
      std::vector<ObjectPtr> refs;
      if ((st = resolve(x, &p[i], &bounds[i], &src, &refs, true))) return fold_fail(x, F, st);
      BatchItem it;
      it.id = bounds[i].id;
      it.src = src;
      it.b = bounds[i];
      it.refs = refs;
      if ((st = plan_star_cached(x, bounds[i], src, refs, &it.plan))) return fold_fail(x, F, st);
      bool eligible = !it.plan.empty_src && !it.plan.needs_prog && !src->host;
      for (int m = 0; m < it.plan.nmet; m++) eligible &= it.plan.wide[m] != 0;
      if (!eligible) {
        if ((st = complete_now(i))) return fold_fail(x, F, st);
        continue;
      }
      groups[src->storage[0].get()].push_back({i, std::move(it)});
    }
    size_t words = 0;  // pinned bounds used so far
    for (auto& g : groups) {
      auto& tagged = g.second;
      std::vector<BatchItem> items;
      for (auto& t : tagged) items.push_back(std::move(t.second));
      const int policy = x->cfg.batch_policy;
      if (policy == SVM_BATCH_NEVER || (policy == SVM_BATCH_AUTO && !batch_is_cheaper(items))) {
        for (auto& t : tagged)
          if ((st = complete_now(t.first))) return fold_fail(x, F, st);
        continue;
      }
      for (size_t b0 = 0; b0 < items.size(); b0 += 1024) {
        const size_t b1 = std::min(items.size(), b0 + 1024);
        std::vector<BatchItem> part(items.begin() + (long)b0, items.begin() + (long)b1);
        FoldPart fp;
        fp.host_off = words;
        if ((st = exec_batch(x, part, &fp, (unsigned long long*)F->bounds.p + words))) return fold_fail(x, F, st);
        words += (size_t)fp.nq + 2;
        const int pi = (int)F->parts.size();
        for (size_t j = 0; j < fp.order.size(); j++) {
          Fold::Res& r = F->res[tagged[b0 + (size_t)fp.order[j]].first];
          r.part = pi;
          r.pos = (int)j;
        }
        F->parts.push_back(std::move(fp));
      }
    }
  }
  cudaError_t e = cudaSuccess;
  if (F->want_host) {
    // Every part's whole store (36 bytes a group), then each completed
    // result's columns in its host layout.
    size_t total = 0;
    for (const FoldPart& fp : F->parts) {
      F->part_stage.push_back(total);
      F->part_groups.push_back(fp.store->nrows);
      total += 36 * (size_t)fp.store->nrows;
    }
    for (Fold::Res& r : F->res) {
      if (!r.done) continue;
      for (int c = 0; c < r.done->ncols; c++)
        if (r.done->is_string(c)) return fold_fail(x, F, x->fail(SVM_E_UNSUPPORTED, "fold read: " + r.id +
                                                                 " has a String column (read it with svm_object_read)"));
      r.stage_off = total;
      total += host_bytes(r.done->types, r.done->nrows);
    }
    if ((st = x->pinned_take(total + 8, &F->stage))) return fold_fail(x, F, st);
    char* stage = (char*)F->stage.p;
    for (size_t pi = 0; pi < F->parts.size() && !e; pi++) {
      const ObjectPtr& all = F->parts[pi].store;
      const size_t G = all->nrows;
      for (int c = 0; c < 6 && !e && G; c++) {
        const size_t off = F->part_stage[pi] + (c < 3 ? 4 * G * c : 12 * G + 8 * G * (c - 3));
        e = cudaMemcpyAsync(stage + off, all->col(c), G * (c < 3 ? 4 : 8), cudaMemcpyDeviceToHost, x->stream);
      }
    }
    for (Fold::Res& r : F->res) {
      if (!r.done || e) continue;
      size_t off = r.stage_off;
      for (int c = 0; c < r.done->ncols && !e; c++) {
        const size_t b = r.done->nrows * r.done->elem(c);
        if (b) e = cudaMemcpyAsync(stage + off, r.done->col(c), b, cudaMemcpyDeviceToHost, x->stream);
        off += (b + 7) & ~size_t(7);
      }
    }
  }
  if (!e) e = cudaEventCreateWithFlags(&F->done, cudaEventDisableTiming);
  if (!e) e = cudaEventRecord(F->done, x->stream);
  if (e) return fold_fail(x, F, x->cuda_fail(e, "fold enqueue"));
  *out = F;
  return SVM_OK;
}

svm_status batch_wait(Ctx* x, void* fold, void* host, unsigned long long cap, unsigned long long* nrows_out,
                      unsigned long long* needed) {
  Fold* F = static_cast<Fold*>(fold);
  cudaError_t e = cudaEventSynchronize(F->done);
  if (e) return x->cuda_fail(e, "fold wait");
  const unsigned long long* hb = (const unsigned long long*)F->bounds.p;
  std::vector<unsigned long long> rows(F->res.size(), 0);
  // Results of the batched parts (their error words first).
  for (size_t pi = 0; pi < F->parts.size(); pi++) {
    FoldPart& fp = F->parts[pi];
    const unsigned long long* b = hb + fp.host_off;
    const int err = (int)(uint32_t)b[fp.nq + 1];
    if (err) {
      const char* m;
      const svm_status s = device_error_status(err, &m);
      return x->fail(s, std::string("batch: ") + m);
    }
    if (!fp.items.empty()) {
      svm_status st = store_batch_results(x, fp.items, fp.order, fp.store, b);
      if (st) return st;
      fp.items.clear();  // results stored once
    }
  }
  unsigned long long total = 0;
  for (size_t i = 0; i < F->res.size(); i++) {
    const Fold::Res& r = F->res[i];
    if (r.part >= 0) {
      const unsigned long long* b = hb + F->parts[r.part].host_off;
      rows[i] = b[r.pos + 1] - b[r.pos];
      ObjectPtr o = x->find(r.id);
      total += o ? host_bytes(o->types, rows[i]) : 0;
    } else if (r.done) {
      rows[i] = r.done->nrows;
      total += host_bytes(r.done->types, rows[i]);
    }
    if (nrows_out) nrows_out[i] = rows[i];
  }
  if (needed) *needed = F->want_host ? total : 0;
  if (!host) return SVM_OK;
  if (!F->want_host) return x->fail(SVM_E_INVALID_ARG, "fold read: results were not staged (want_host 0)");
  if (cap < total) return x->fail(SVM_E_INVALID_ARG, "fold read: host buffer smaller than needed bytes");
  char* out = (char*)host;
  const char* stage = (const char*)F->stage.p;
  for (size_t i = 0; i < F->res.size(); i++) {
    const Fold::Res& r = F->res[i];
    if (r.part >= 0) {
      const unsigned long long* b = hb + F->parts[r.part].host_off;
      const unsigned long long row0 = b[r.pos], G = F->part_groups[r.part];
      ObjectPtr o = x->find(r.id);
      const int nk = (int)std::count(o->types.begin(), o->types.end(), SVM_INT32);
      const size_t base = F->part_stage[r.part];
      for (int c = 0; c < o->ncols; c++) {
        const bool key = c < nk;
        const size_t col = key ? (size_t)c : 3 + (size_t)(c - nk);
        const size_t w = key ? 4 : 8;
        const size_t off = base + (col < 3 ? 4 * G * col : 12 * G + 8 * G * (col - 3)) + w * row0;
        std::memcpy(out, stage + off, w * rows[i]);
        out += (w * rows[i] + 7) & ~size_t(7);
      }
    } else if (r.done) {
      const size_t b = host_bytes(r.done->types, rows[i]);
      std::memcpy(out, stage + r.stage_off, b);
      out += b;
    }
  }
  return SVM_OK;
}

void Ctx::forget_plans(const Object* o) {
  if (!plan_cache) return;
  PlanCache* pc = static_cast<PlanCache*>(plan_cache.get());
  auto f = pc->by_object.find(o);
  if (f == pc->by_object.end()) return;
  for (const std::string& k : f->second) pc->plans.erase(k);
  pc->by_object.erase(f);
}

void fold_sync(void* fold) {
  Fold* F = static_cast<Fold*>(fold);
  if (F && F->done) cudaEventSynchronize(F->done);
}

void batch_discard(Ctx* x, void* fold) {
  Fold* F = static_cast<Fold*>(fold);
  if (!F) return;
  if (F->done) cudaEventSynchronize(F->done);
  x->pinned_give(&F->bounds);
  x->pinned_give(&F->stage);
  if (F->done) cudaEventDestroy(F->done);
  delete F;
}

}  // namespace svm
