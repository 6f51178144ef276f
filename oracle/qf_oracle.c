/*
 * qf_oracle.c -- CPU oracle (test infrastructure only; see qf_oracle.h).
 *
 * A plain-C restatement of the reference's candidate-literal operator chain:
 * RadixPartition -> BuildHashTableOnPartitions -> PartitionAssigner/HashJoin
 * -> Filter -> CountAggregator, plus the semi-joins and the label-aware
 * binding-set extension.  The data structures follow the reference exactly
 * (8-byte partition tuples, 1-based chained buckets, per-binding-partition
 * semi bit vectors) so that the CPU baseline does the same work the
 * reference does.
 */
#include "qf_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Hashing: utility/Hash.hpp:16-55.  Hash(int32) is std::hash<int>, which is
 * the identity in libstdc++, cast to uint32. */
static inline uint32_t hash_i32(int32_t v) { return (uint32_t)v; }

static inline uint32_t hash_combine(uint32_t seed, int32_t v) {
  return seed ^ (hash_i32(v) + 0x9e3779b9u + (seed << 6) + (seed >> 2));
}

static int keys_equal(const int32_t* const* a, int64_t ta, const int32_t* const* b, int64_t tb,
                      int num_keys);

uint32_t qfo_hash_keys(const int32_t* const* keys, int num_keys, int64_t tid) {
  uint32_t seed = hash_i32(keys[0][tid]);
  for (int i = 1; i < num_keys; ++i) seed = hash_combine(seed, keys[i][tid]);
  return seed;
}

/* storage/FoilHashTable.cpp:17-31 (NEXT_POW_2) and :34-49. */
int32_t qfo_num_buckets(int32_t n) {
  uint32_t v = (uint32_t)n;
  v--;
  v |= v >> 1;
  v |= v >> 2;
  v |= v >> 4;
  v |= v >> 8;
  v |= v >> 16;
  v++;
  return (int32_t)v;
}

/* ------------------------------------------------------------------------ */
/* operations/RadixPartition.cpp:56-155.  The reference builds a histogram,
 * then scatters through cache-line write-combining buffers; the visible
 * result is a stable partition by the low radix bits of the identity hash. */
void qfo_radix_partition(const int32_t* values, int64_t n, int bits,
                         qfo_partition_tuple* out, int64_t* offsets) {
  const int64_t num_partitions = (int64_t)1 << bits;
  const uint32_t mask = (uint32_t)(num_partitions - 1);
  int64_t* cursor = (int64_t*)calloc((size_t)num_partitions, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) cursor[hash_i32(values[i]) & mask]++;
  int64_t acc = 0;
  for (int64_t p = 0; p < num_partitions; ++p) {
    offsets[p] = acc;
    acc += cursor[p];
    cursor[p] = offsets[p];
  }
  offsets[num_partitions] = acc;
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t p = hash_i32(values[i]) & mask;
    qfo_partition_tuple* t = &out[cursor[p]++];
    t->value = values[i];
    t->tuple_id = (int32_t)i;
  }
  free(cursor);
}

/* operations/BuildHashTable.cpp:54-93: insert in partition order, each new
 * tuple becomes the chain head (1-based), so a chain lists positions in
 * descending order. */
uint32_t qfo_build_partition_hash_table(const qfo_partition_tuple* part, int32_t n,
                                        int bits, int32_t* buckets, int32_t* next) {
  const int32_t nb = qfo_num_buckets(n);
  const uint32_t mask = ((uint32_t)nb - 1u) << bits;
  memset(buckets, 0, sizeof(int32_t) * (size_t)nb);
  for (int32_t i = 0; i < n; ++i) {
    const uint32_t bucket = (hash_i32(part[i].value) & mask) >> bits;
    next[i] = buckets[bucket];
    buckets[bucket] = i + 1;
  }
  return mask;
}

/* operations/BuildHashTable.cpp:97-125 (radix bits 0). */
uint32_t qfo_build_table_hash_table(const int32_t* const* keys, int num_keys, int64_t n,
                                    int32_t* buckets, int32_t* next) {
  const int32_t nb = qfo_num_buckets((int32_t)n);
  const uint32_t mask = (uint32_t)nb - 1u;
  memset(buckets, 0, sizeof(int32_t) * (size_t)nb);
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t bucket = qfo_hash_keys(keys, num_keys, i) & mask;
    next[i] = buckets[bucket];
    buckets[bucket] = (int32_t)i + 1;
  }
  return mask;
}

/* operations/BuildHashTable.cpp:127-189 (InsertIfNotPresent,
 * BuildHashTableAfterSemiJoinImpl) with the chunking of
 * operations/LeftSemiJoin.hpp:55-83; see qf_oracle.h. */
static uint32_t after_semijoin_readable(const int32_t* const* keys, int num_keys, int64_t num_rows,
                                        int64_t readable, const uint64_t* bits, int64_t chunk_rows,
                                        int32_t num_build_tuples, int32_t* buckets, int32_t* next);

uint32_t qfo_build_hash_table_after_semijoin(const int32_t* const* keys, int num_keys,
                                             int64_t num_rows, const uint64_t* bits,
                                             int64_t chunk_rows, int32_t num_build_tuples,
                                             int32_t* buckets, int32_t* next) {
  return after_semijoin_readable(keys, num_keys, num_rows, num_rows, bits, chunk_rows,
                                 num_build_tuples, buckets, next);
}

/* As above; the columns go on past the last row up to `readable` rows,
 * where a chain position of a short last chunk is read (beyond: unequal). */
static uint32_t after_semijoin_readable(const int32_t* const* keys, int num_keys, int64_t num_rows,
                                        int64_t readable, const uint64_t* bits, int64_t chunk_rows,
                                        int32_t num_build_tuples, int32_t* buckets, int32_t* next) {
  const int32_t nb = qfo_num_buckets(num_build_tuples);
  const uint32_t mask = (uint32_t)nb - 1u;
  memset(buckets, 0, sizeof(int32_t) * (size_t)nb);
  memset(next, 0, sizeof(int32_t) * (size_t)num_build_tuples);
  if (chunk_rows <= 0 || chunk_rows > num_rows) chunk_rows = num_rows;
  const int32_t* chunk_keys[QFO_MAX_ARITY];
  for (int64_t c0 = 0; c0 < num_rows; c0 += chunk_rows) {
    const int64_t len = num_rows - c0 < chunk_rows ? num_rows - c0 : chunk_rows;
    for (int k = 0; k < num_keys; ++k) chunk_keys[k] = keys[k] + c0;
    for (int64_t tid = 0; tid < len; ++tid) {
      const int64_t row = c0 + tid;
      if (!((bits[row >> 6] >> (row & 63)) & 1u)) continue;
      const uint32_t bucket = qfo_hash_keys(chunk_keys, num_keys, tid) & mask;
      int exist = 0;
      for (int32_t pos = buckets[bucket] - 1; pos >= 0; pos = next[pos] - 1) {
        /* A position an earlier, longer chunk inserted can lie past the end
         * of a short last chunk: the reference then reads on past the end of
         * the columns.  Here such a position is read while the columns go
         * on (`readable`) and compares unequal beyond. */
        if (c0 + pos < readable && keys_equal(chunk_keys, tid, chunk_keys, pos, num_keys)) {
          exist = 1;
          break;
        }
      }
      if (!exist) {
        next[tid] = buckets[bucket];
        buckets[bucket] = (int32_t)tid + 1;
      }
    }
  }
  return mask;
}

/* ------------------------------------------------------------------------ */
/* A partitioned column with its per-partition chained hash tables
 * (TableView::partitions_ + hash_tables_, storage/TableView.hpp:62-80). */
typedef struct {
  const int32_t* column;   /* identity of the source column (cache key) */
  int64_t n;
  int bits;
  qfo_partition_tuple* tuples;
  int64_t* offsets;        /* 2^bits + 1 */
  int64_t* bucket_offsets; /* start of partition p's buckets in buckets[] */
  int32_t* buckets;
  int32_t* next;           /* indexed like tuples (partition-relative chains) */
  uint32_t* masks;
} partitioned_column;

static void partitioned_column_free(partitioned_column* pc) {
  if (pc == NULL) return;
  free(pc->tuples);
  free(pc->offsets);
  free(pc->bucket_offsets);
  free(pc->buckets);
  free(pc->next);
  free(pc->masks);
  free(pc);
}

static partitioned_column* partition_column(const int32_t* column, int64_t n, int bits,
                                            int with_hash_tables) {
  const int64_t np = (int64_t)1 << bits;
  partitioned_column* pc = (partitioned_column*)calloc(1, sizeof(partitioned_column));
  pc->column = column;
  pc->n = n;
  pc->bits = bits;
  pc->tuples = (qfo_partition_tuple*)malloc(sizeof(qfo_partition_tuple) * (size_t)(n > 0 ? n : 1));
  pc->offsets = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np + 1));
  qfo_radix_partition(column, n, bits, pc->tuples, pc->offsets);
  if (with_hash_tables) {
    pc->bucket_offsets = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np + 1));
    pc->masks = (uint32_t*)calloc((size_t)np, sizeof(uint32_t));
    int64_t total = 0;
    for (int64_t p = 0; p < np; ++p) {
      pc->bucket_offsets[p] = total;
      const int64_t cnt = pc->offsets[p + 1] - pc->offsets[p];
      if (cnt > 0) total += qfo_num_buckets((int32_t)cnt);
    }
    pc->bucket_offsets[np] = total;
    pc->buckets = (int32_t*)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    pc->next = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t p = 0; p < np; ++p) {
      const int64_t cnt = pc->offsets[p + 1] - pc->offsets[p];
      if (cnt == 0) continue; /* BuildHashTable.cpp:66-69: empty partition, empty table */
      pc->masks[p] = qfo_build_partition_hash_table(pc->tuples + pc->offsets[p], (int32_t)cnt,
                                                    bits, pc->buckets + pc->bucket_offsets[p],
                                                    pc->next + pc->offsets[p]);
    }
  }
  return pc;
}

/* ------------------------------------------------------------------------ */
struct qfo_relcache {
  int size, cap;
  partitioned_column** entries;
  pthread_mutex_t lock;
};

qfo_relcache* qfo_relcache_create(void) {
  qfo_relcache* c = (qfo_relcache*)calloc(1, sizeof(qfo_relcache));
  pthread_mutex_init(&c->lock, NULL);
  return c;
}

void qfo_relcache_destroy(qfo_relcache* c) {
  if (c == NULL) return;
  for (int i = 0; i < c->size; ++i) partitioned_column_free(c->entries[i]);
  free(c->entries);
  pthread_mutex_destroy(&c->lock);
  free(c);
}

static partitioned_column* relcache_get(qfo_relcache* c, const int32_t* column, int64_t n,
                                        int bits) {
  for (int i = 0; i < c->size; ++i) {
    partitioned_column* e = c->entries[i];
    if (e->column == column && e->n == n && e->bits == bits) return e;
  }
  partitioned_column* e = partition_column(column, n, bits, 0);
  if (c->size == c->cap) {
    c->cap = c->cap ? 2 * c->cap : 16;
    c->entries = (partitioned_column**)realloc(c->entries, sizeof(*c->entries) * (size_t)c->cap);
  }
  c->entries[c->size++] = e;
  return e;
}

/* ------------------------------------------------------------------------ */
/* One work item = (literal, partition).  The reference's PartitionAssigner
 * (operations/PartitionAssigner.hpp:77-138) walks partition -> relation ->
 * join group -> 32768-tuple chunks; HashJoin::Next (operations/HashJoin.cpp:
 * 23-86) probes the binding partition's chained table with every relation
 * tuple of the chunk; Filter::Next (operations/Filter.cpp:17-38) evaluates
 * each atom R[pos] == B[var] over the join pairs; CountAggregator
 * (operations/CountAggregator.cpp:111-243) adds one binding count per
 * passing pair and one covered count per binding row whose semi bit
 * (indexed by its position inside the binding partition, reset per
 * partition :121-125) was not yet set.  Chunking does not change the counts,
 * so each item walks its whole relation partition.  The shared-conjunction
 * plan (learner/CandidateLiteralEvaluator.cpp:105-262) only shares ANDs
 * between literals; a literal's pass bit is the AND of its own atoms. */
typedef struct {
  const qfo_table* relations;
  const qfo_table* bindings;
  int64_t num_positive;
  const qfo_literal* literals;
  partitioned_column** rel_parts;  /* per literal */
  partitioned_column** bind_parts; /* per literal */
  int num_partitions;
  int64_t num_items;
  int64_t next_item;
  int64_t* item_counts;            /* 4 per item */
  pthread_mutex_t lock;
  int64_t max_binding_partition;
} eval_job;

static void eval_item(eval_job* job, int64_t item, uint64_t* semi) {
  const int lit_index = (int)(item / job->num_partitions);
  const int p = (int)(item % job->num_partitions);
  const qfo_literal* lit = &job->literals[lit_index];
  const partitioned_column* rp = job->rel_parts[lit_index];
  const partitioned_column* bp = job->bind_parts[lit_index];
  int64_t* out = &job->item_counts[4 * item];
  out[0] = out[1] = out[2] = out[3] = 0;

  const int64_t b_begin = bp->offsets[p], b_end = bp->offsets[p + 1];
  const int64_t r_begin = rp->offsets[p], r_end = rp->offsets[p + 1];
  if (b_end == b_begin || r_end == r_begin) return; /* HashJoin.cpp:37-39 */

  const qfo_partition_tuple* btup = bp->tuples + b_begin;
  const int32_t* buckets = bp->buckets + bp->bucket_offsets[p];
  const int32_t* next = bp->next + b_begin;
  const uint32_t mask = bp->masks[p];
  const int bits = bp->bits;

  /* Atoms: every bound argument other than the join key. */
  int num_atoms = 0;
  const int32_t* atom_rel[QFO_MAX_ARITY];
  const int32_t* atom_bind[QFO_MAX_ARITY];
  const qfo_table* rel = &job->relations[lit->relation];
  for (int k = 0; k < lit->num_args; ++k) {
    if (k == lit->join_pos || lit->vars[k] < 0) continue;
    atom_rel[num_atoms] = rel->columns[k];
    atom_bind[num_atoms] = job->bindings->columns[lit->vars[k]];
    ++num_atoms;
  }

  const int64_t nb = b_end - b_begin;
  memset(semi, 0, sizeof(uint64_t) * (size_t)((nb + 63) / 64));
  const int64_t P = job->num_positive;
  for (int64_t ri = r_begin; ri < r_end; ++ri) {
    const int32_t v = rp->tuples[ri].value;
    const int32_t r = rp->tuples[ri].tuple_id;
    const uint32_t bucket = (hash_i32(v) & mask) >> bits;
    for (int32_t pos = buckets[bucket] - 1; pos >= 0; pos = next[pos] - 1) {
      if (btup[pos].value != v) continue;
      const int32_t b = btup[pos].tuple_id;
      int pass = 1;
      for (int a = 0; a < num_atoms; ++a) {
        if (atom_rel[a][r] != atom_bind[a][b]) {
          pass = 0;
          break;
        }
      }
      if (!pass) continue;
      const int neg = (b >= P);
      out[2 + neg] += 1;
      const uint64_t bit = (uint64_t)1 << (pos & 63);
      if (!(semi[pos >> 6] & bit)) {
        semi[pos >> 6] |= bit;
        out[neg] += 1;
      }
    }
  }
}

static void* eval_worker(void* arg) {
  eval_job* job = (eval_job*)arg;
  uint64_t* semi =
      (uint64_t*)malloc(sizeof(uint64_t) * (size_t)((job->max_binding_partition + 63) / 64 + 1));
  for (;;) {
    pthread_mutex_lock(&job->lock);
    const int64_t item = job->next_item++;
    pthread_mutex_unlock(&job->lock);
    if (item >= job->num_items) break;
    eval_item(job, item, semi);
  }
  free(semi);
  return NULL;
}

int qfo_evaluate(qfo_relcache* cache, const qfo_table* relations, int num_relations,
                 const qfo_table* bindings, int64_t num_positive,
                 const qfo_literal* literals, int num_literals, int bits, int nthreads,
                 int64_t* counts) {
  if (bits < 1 || bits > 24 || num_literals < 0) return 1;
  for (int i = 0; i < num_literals; ++i) {
    const qfo_literal* l = &literals[i];
    if (l->relation < 0 || l->relation >= num_relations) return 1;
    if (l->num_args < 1 || l->num_args > QFO_MAX_ARITY) return 1;
    if (l->num_args > relations[l->relation].num_columns) return 1;
    if (l->join_pos < 0 || l->join_pos >= l->num_args || l->vars[l->join_pos] < 0) return 1;
    for (int k = 0; k < l->num_args; ++k)
      if (l->vars[k] >= bindings->num_columns) return 1;
  }
  memset(counts, 0, sizeof(int64_t) * 4 * (size_t)num_literals);
  if (num_literals == 0) return 0;

  /* Binding partitions + hash tables, once per distinct join column
   * (learner/CandidateLiteralEvaluator.cpp:316-323). */
  partitioned_column** bind_by_col =
      (partitioned_column**)calloc((size_t)bindings->num_columns, sizeof(partitioned_column*));
  eval_job job;
  memset(&job, 0, sizeof(job));
  job.relations = relations;
  job.bindings = bindings;
  job.num_positive = num_positive;
  job.literals = literals;
  job.num_partitions = 1 << bits;
  job.rel_parts = (partitioned_column**)calloc((size_t)num_literals, sizeof(partitioned_column*));
  job.bind_parts = (partitioned_column**)calloc((size_t)num_literals, sizeof(partitioned_column*));
  for (int i = 0; i < num_literals; ++i) {
    const qfo_literal* l = &literals[i];
    const int j = l->vars[l->join_pos];
    if (bind_by_col[j] == NULL)
      bind_by_col[j] = partition_column(bindings->columns[j], bindings->num_tuples, bits, 1);
    job.bind_parts[i] = bind_by_col[j];
    const qfo_table* rel = &relations[l->relation];
    job.rel_parts[i] = relcache_get(cache, rel->columns[l->join_pos], rel->num_tuples, bits);
  }
  for (int j = 0; j < bindings->num_columns; ++j) {
    if (bind_by_col[j] == NULL) continue;
    for (int p = 0; p < job.num_partitions; ++p) {
      const int64_t c = bind_by_col[j]->offsets[p + 1] - bind_by_col[j]->offsets[p];
      if (c > job.max_binding_partition) job.max_binding_partition = c;
    }
  }
  job.num_items = (int64_t)num_literals * job.num_partitions;
  job.item_counts = (int64_t*)malloc(sizeof(int64_t) * 4 * (size_t)job.num_items);
  pthread_mutex_init(&job.lock, NULL);
  if (nthreads <= 1) {
    eval_worker(&job);
  } else {
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, eval_worker, &job);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
  }
  pthread_mutex_destroy(&job.lock);
  for (int64_t it = 0; it < job.num_items; ++it) {
    const int lit = (int)(it / job.num_partitions);
    for (int c = 0; c < 4; ++c) counts[4 * lit + c] += job.item_counts[4 * it + c];
  }
  for (int j = 0; j < bindings->num_columns; ++j) partitioned_column_free(bind_by_col[j]);
  free(bind_by_col);
  free(job.rel_parts);
  free(job.bind_parts);
  free(job.item_counts);
  return 0;
}

/* ------------------------------------------------------------------------ */
static int keys_equal(const int32_t* const* a, int64_t ta, const int32_t* const* b, int64_t tb,
                      int num_keys) {
  for (int i = 0; i < num_keys; ++i)
    if (a[i][ta] != b[i][tb]) return 0;
  return 1;
}

int64_t qfo_left_semijoin(const int32_t* const* probe_keys, int64_t num_probe,
                          const int32_t* const* build_keys, int64_t num_build, int num_keys,
                          uint64_t* out_bits) {
  memset(out_bits, 0, sizeof(uint64_t) * (size_t)((num_probe + 63) / 64));
  if (num_build == 0) return 0;
  const int32_t nb = qfo_num_buckets((int32_t)num_build);
  int32_t* buckets = (int32_t*)malloc(sizeof(int32_t) * (size_t)nb);
  int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)num_build);
  const uint32_t mask = qfo_build_table_hash_table(build_keys, num_keys, num_build, buckets, next);
  int64_t ones = 0;
  for (int64_t t = 0; t < num_probe; ++t) {
    const uint32_t bucket = qfo_hash_keys(probe_keys, num_keys, t) & mask;
    for (int32_t pos = buckets[bucket] - 1; pos >= 0; pos = next[pos] - 1) {
      if (keys_equal(probe_keys, t, build_keys, pos, num_keys)) {
        out_bits[t >> 6] |= (uint64_t)1 << (t & 63);
        ++ones;
        break;
      }
    }
  }
  free(buckets);
  free(next);
  return ones;
}

int64_t qfo_right_semijoin(const int32_t* const* probe_keys, int64_t num_probe,
                           const int32_t* const* build_keys, int64_t num_build, int num_keys,
                           uint64_t* out_bits) {
  memset(out_bits, 0, sizeof(uint64_t) * (size_t)((num_build + 63) / 64));
  if (num_build == 0) return 0;
  const int32_t nb = qfo_num_buckets((int32_t)num_build);
  int32_t* buckets = (int32_t*)malloc(sizeof(int32_t) * (size_t)nb);
  int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)num_build);
  const uint32_t mask = qfo_build_table_hash_table(build_keys, num_keys, num_build, buckets, next);
  int64_t ones = 0;
  for (int64_t t = 0; t < num_probe; ++t) {
    const uint32_t bucket = qfo_hash_keys(probe_keys, num_keys, t) & mask;
    for (int32_t pos = buckets[bucket] - 1; pos >= 0; pos = next[pos] - 1) {
      if (keys_equal(probe_keys, t, build_keys, pos, num_keys)) {
        const uint64_t bit = (uint64_t)1 << (pos & 63);
        if (!(out_bits[pos >> 6] & bit)) {
          out_bits[pos >> 6] |= bit;
          ++ones;
        }
      }
    }
  }
  free(buckets);
  free(next);
  return ones;
}

/* ------------------------------------------------------------------------ */
/* MultiColumnHashJoin::DoBlockJoin (operations/MultiColumnHashJoin.cpp:
 * 496-528) over a whole probe side: for each probe row in order, every build
 * row with equal keys in chain order (descending build index).  Calls emit()
 * per pair; the join chunking (:432-486) does not change the order. */
typedef void (*emit_fn)(void* ctx, int64_t probe_tid, int64_t build_tid);

static void block_join(const int32_t* const* probe_keys, int64_t num_probe,
                       const int32_t* const* build_keys, int64_t num_build, int num_keys,
                       emit_fn emit, void* ctx) {
  if (num_build == 0 || num_probe == 0) return;
  const int32_t nb = qfo_num_buckets((int32_t)num_build);
  int32_t* buckets = (int32_t*)malloc(sizeof(int32_t) * (size_t)nb);
  int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)num_build);
  const uint32_t mask = qfo_build_table_hash_table(build_keys, num_keys, num_build, buckets, next);
  for (int64_t t = 0; t < num_probe; ++t) {
    const uint32_t bucket = qfo_hash_keys(probe_keys, num_keys, t) & mask;
    for (int32_t pos = buckets[bucket] - 1; pos >= 0; pos = next[pos] - 1)
      if (keys_equal(probe_keys, t, build_keys, pos, num_keys)) emit(ctx, t, pos);
  }
  free(buckets);
  free(next);
}

typedef struct {
  int num_clause_columns;
  int num_unbound;
  const int32_t* const* clause_cols; /* this label's binding columns, row 0 = label start */
  const int32_t* unbound_rel_cols[QFO_MAX_ARITY];
  int relation_is_probe;
  int32_t* const* out;
  int64_t out_base, out_limit, produced;
} extend_ctx;

static void extend_emit(void* vctx, int64_t probe_tid, int64_t build_tid) {
  extend_ctx* c = (extend_ctx*)vctx;
  const int64_t b = c->relation_is_probe ? build_tid : probe_tid;
  const int64_t r = c->relation_is_probe ? probe_tid : build_tid;
  if (c->produced < c->out_limit) {
    const int64_t row = c->out_base + c->produced;
    for (int i = 0; i < c->num_clause_columns; ++i) c->out[i][row] = c->clause_cols[i][b];
    for (int u = 0; u < c->num_unbound; ++u)
      c->out[c->num_clause_columns + u][row] = c->unbound_rel_cols[u][r];
  }
  c->produced++;
}

int qfo_extend_bindings(const qfo_table* bindings, int64_t num_positive,
                        const qfo_table* relation, const qfo_literal* literal,
                        int64_t num_out_positive, int64_t num_out_negative,
                        int32_t* const* out_columns) {
  const int nc = bindings->num_columns;
  const int64_t P = num_positive, N = bindings->num_tuples - num_positive;
  const int32_t* rel_keys[QFO_MAX_ARITY];
  const int32_t* pos_keys[QFO_MAX_ARITY];
  const int32_t* neg_keys[QFO_MAX_ARITY];
  const int32_t* pos_cols[64];
  const int32_t* neg_cols[64];
  if (nc > 64) return 2;
  int nk = 0;
  extend_ctx c;
  memset(&c, 0, sizeof(c));
  c.num_clause_columns = nc;
  for (int i = 0; i < nc; ++i) {
    pos_cols[i] = bindings->columns[i];
    neg_cols[i] = bindings->columns[i] + P;
  }
  /* operations/MultiColumnHashJoin.cpp:132-141: bound arguments are keys,
   * unbound arguments become new binding columns. */
  for (int k = 0; k < literal->num_args; ++k) {
    if (literal->vars[k] >= 0) {
      rel_keys[nk] = relation->columns[k];
      pos_keys[nk] = bindings->columns[literal->vars[k]];
      neg_keys[nk] = bindings->columns[literal->vars[k]] + P;
      ++nk;
    } else {
      c.unbound_rel_cols[c.num_unbound++] = relation->columns[k];
    }
  }
  c.out = out_columns;
  const int64_t R = relation->num_tuples;
  int64_t produced_pos, produced_neg;
  /* :172-207 probe with the relation when both label sides are smaller
   * than it (CollaborateJoin); :208-250 otherwise build on the relation and
   * probe with the positives, then the negatives. */
  c.relation_is_probe = (P < R && N < R);
  c.clause_cols = pos_cols;
  c.out_base = 0;
  c.out_limit = num_out_positive;
  c.produced = 0;
  if (c.relation_is_probe)
    block_join(rel_keys, R, pos_keys, P, nk, extend_emit, &c);
  else
    block_join(pos_keys, P, rel_keys, R, nk, extend_emit, &c);
  produced_pos = c.produced;
  c.clause_cols = neg_cols;
  c.out_base = num_out_positive;
  c.out_limit = num_out_negative;
  c.produced = 0;
  if (c.relation_is_probe)
    block_join(rel_keys, R, neg_keys, N, nk, extend_emit, &c);
  else
    block_join(neg_keys, N, rel_keys, R, nk, extend_emit, &c);
  produced_neg = c.produced;
  return (produced_pos == num_out_positive && produced_neg == num_out_negative) ? 0 : 3;
}

int qfo_coverage(const qfo_table* bindings, int64_t num_positive, const qfo_table* relation,
                 const qfo_literal* literal, int num_target_columns,
                 const qfo_table* uncovered_positive, const qfo_table* negative,
                 uint64_t* positive_bits, int64_t* num_covered) {
  const int k = num_target_columns;
  if (literal->num_args != relation->num_columns || k < 1 || k > QFO_MAX_ARITY ||
      k > bindings->num_columns)
    return 1;
  const int32_t* rel_keys[QFO_MAX_ARITY];
  int bound_vars[QFO_MAX_ARITY];
  int nk = 0;
  for (int a = 0; a < literal->num_args; ++a) {
    const int v = literal->vars[a];
    if (v >= bindings->num_columns || v < -1) return 1;
    if (v < 0) continue;
    rel_keys[nk] = relation->columns[a];
    bound_vars[nk++] = v;
  }
  if (nk == 0) return 1;
  num_covered[0] = num_covered[1] = 0;
  const int64_t nu = uncovered_positive != NULL ? uncovered_positive->num_tuples : 0;
  if (positive_bits != NULL) memset(positive_bits, 0, sizeof(uint64_t) * (size_t)((nu + 63) / 64));
  for (int label = 0; label < 2; ++label) {
    const qfo_table* ex = label == 0 ? uncovered_positive : negative;
    if (ex == NULL || ex->num_tuples == 0) continue;
    const int64_t lo = label == 0 ? 0 : num_positive;
    const int64_t n = label == 0 ? num_positive : bindings->num_tuples - num_positive;
    /* binding semi-join: the side's rows against the relation (:515-522) */
    const int32_t* side_keys[QFO_MAX_ARITY];
    for (int q = 0; q < nk; ++q) side_keys[q] = bindings->columns[bound_vars[q]] + lo;
    uint64_t* pass = (uint64_t*)calloc((size_t)((n + 63) / 64) + 1, sizeof(uint64_t));
    const int64_t npass = qfo_left_semijoin(side_keys, n, rel_keys, relation->num_tuples, nk, pass);
    /* the passing rows' target tuples (:523-526) */
    int32_t* proj[QFO_MAX_ARITY];
    for (int q = 0; q < k; ++q) proj[q] = (int32_t*)malloc(sizeof(int32_t) * (size_t)(npass + 1));
    int64_t m = 0;
    for (int64_t r = 0; r < n; ++r) {
      if (!(pass[r >> 6] >> (r & 63) & 1)) continue;
      for (int q = 0; q < k; ++q) proj[q][m] = bindings->columns[q][lo + r];
      ++m;
    }
    /* coverage semi-join: the examples against the projections (:528-541) */
    uint64_t* bits = label == 0 && positive_bits != NULL
                         ? positive_bits
                         : (uint64_t*)calloc((size_t)((ex->num_tuples + 63) / 64) + 1,
                                             sizeof(uint64_t));
    num_covered[label] = qfo_left_semijoin(ex->columns, ex->num_tuples,
                                           (const int32_t* const*)proj, m, k, bits);
    if (bits != positive_bits) free(bits);
    for (int q = 0; q < k; ++q) free(proj[q]);
    free(pass);
  }
  return 0;
}

int64_t qfo_compact_rows(int num_columns, const int32_t* const* columns, int64_t n,
                         const uint64_t* bits, int keep_set, int32_t* const* out) {
  int64_t m = 0;
  for (int64_t r = 0; r < n; ++r) {
    const int set = (int)(bits[r >> 6] >> (r & 63) & 1);
    if (set != (keep_set != 0)) continue;
    for (int c = 0; c < num_columns; ++c) out[c][m] = columns[c][r];
    ++m;
  }
  return m;
}

static int c_space(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

/* std::stoi on [s, e): 0, or 3 (no digits) / 4 (out of int32). */
static int stoi_field(const char* s, const char* e, int32_t* out) {
  while (s < e && c_space(*s)) ++s;
  int neg = 0;
  if (s < e && (*s == '+' || *s == '-')) {
    neg = *s == '-';
    ++s;
  }
  if (s >= e || *s < '0' || *s > '9') return 3;
  uint64_t v = 0;
  int over = 0;
  for (; s < e && *s >= '0' && *s <= '9'; ++s) {
    if (!over) {
      v = v * 10 + (uint64_t)(*s - '0');
      over = v > 2147483648ull;
    }
  }
  if (over || (!neg && v > 2147483647ull)) return 4;
  *out = neg ? (int32_t)(-(int64_t)v) : (int32_t)v;
  return 0;
}

int qfo_parse_text(const char* text, int64_t n, int num_args, const int32_t* skipped,
                   int32_t* const* out, int64_t capacity, int64_t* num_rows,
                   int64_t* error_line) {
  int64_t rows = 0, line = 0;
  *error_line = 0;
  const char* p = text;
  const char* end = text + n;
  while (p < end) {
    const char* e = memchr(p, '\n', (size_t)(end - p));
    if (e == NULL) e = end;
    ++line;
    if (e > p && *p != '#') {
      int nf = 1;
      for (const char* q = p; q < e; ++q) nf += *q == '|';
      if (nf != num_args) {
        *error_line = line;
        *num_rows = rows;
        return 2;
      }
      int field = 0, col = 0;
      const char* fs = p;
      for (const char* q = p; q <= e; ++q) {
        if (q < e && *q != '|') continue;
        if (!(skipped != NULL && skipped[field])) {
          int32_t v = 0;
          const int rc = stoi_field(fs, q, &v);
          if (rc != 0) {
            *error_line = line;
            *num_rows = rows;
            return rc;
          }
          if (rows < capacity) out[col][rows] = v;
          ++col;
        }
        ++field;
        fs = q + 1;
      }
      ++rows;
    }
    p = e + 1;
  }
  *num_rows = rows;
  return rows > capacity ? 1 : 0;
}


/* QuickFoil::ComputeCoverageOnUncoveredData (learner/QuickFoil.cpp:471-573)
 * step by step as the reference runs it; see qf_oracle.h. */
int qfo_coverage_compat(const qfo_table* bindings, int64_t num_positive, const qfo_table* relation,
                        const qfo_literal* literal, int num_target_columns,
                        const qfo_table* uncovered_positive, const qfo_table* negative,
                        uint64_t* positive_bits, int64_t* num_covered) {
  const int64_t nb = bindings->num_tuples, P = num_positive;
  const int k = num_target_columns;
  const int32_t* rel_keys[QFO_MAX_ARITY];
  const int32_t* bind_keys[QFO_MAX_ARITY];
  int nk = 0;
  for (int i = 0; i < literal->num_args; ++i) {
    if (literal->vars[i] < 0) continue;
    if (literal->vars[i] >= bindings->num_columns) return 1;
    rel_keys[nk] = relation->columns[i];
    bind_keys[nk] = bindings->columns[literal->vars[i]];
    ++nk;
  }
  if (nk == 0 || k < 1 || k > bindings->num_columns) return 1;
  num_covered[0] = num_covered[1] = 0;
  const qfo_table* ex_tab[2] = {uncovered_positive, negative};
  if (positive_bits != NULL && uncovered_positive != NULL)
    memset(positive_bits, 0, sizeof(uint64_t) * (size_t)((uncovered_positive->num_tuples + 63) / 64));
  const int64_t start[2] = {0, P}, rows_of[2] = {P, nb - P};
  for (int s = 0; s < 2; ++s) {
    const int64_t rows = rows_of[s];
    const qfo_table* ex = ex_tab[s];
    if (rows == 0 || ex == NULL || ex->num_tuples == 0 || relation->num_tuples == 0) continue;
    /* First semi-join: the side's rows against the relation (membership). */
    const int32_t* probe[QFO_MAX_ARITY];
    const int32_t* target[QFO_MAX_ARITY];
    for (int q = 0; q < nk; ++q) probe[q] = bind_keys[q] + start[s];
    for (int q = 0; q < k; ++q) target[q] = bindings->columns[q] + start[s];
    uint64_t* member = calloc((size_t)((rows + 63) / 64), sizeof(uint64_t));
    qfo_left_semijoin(probe, rows, rel_keys, relation->num_tuples, nk, member);
    /* SelectAndCreateSemiJoin (operations/SemiJoinFactory.cpp:45-82): one
     * chunk (right semi-join) when the side is smaller than the relation,
     * else 32768-row chunks (FLAGS_semijoin_chunck_size).  The positive side
     * is a view of the consecutive binding columns: reads past its end land
     * on the negative rows. */
    const int64_t chunk = rows < relation->num_tuples ? 0 : 32768;
    const int64_t readable = s == 0 ? nb : rows;
    const int32_t nbt = (int32_t)rows;
    const int32_t nbk = qfo_num_buckets(nbt);
    int32_t* buckets = malloc(sizeof(int32_t) * (size_t)nbk);
    int32_t* next = malloc(sizeof(int32_t) * (size_t)nbt);
    const uint32_t mask = after_semijoin_readable(target, k, rows, readable, member, chunk, nbt,
                                                  buckets, next);
    /* Second semi-join: the examples probed through that table against the
     * side's rows (LeftSemiJoin::DoSemiJoin, operations/LeftSemiJoin.hpp:
     * 86-141). */
    for (int64_t e = 0; e < ex->num_tuples; ++e) {
      const uint32_t b = qfo_hash_keys(ex->columns, k, e) & mask;
      for (int32_t pos = buckets[b] - 1; pos >= 0; pos = next[pos] - 1) {
        if (keys_equal(ex->columns, e, target, pos, k)) {
          ++num_covered[s];
          if (s == 0 && positive_bits != NULL) positive_bits[e >> 6] |= (uint64_t)1 << (e & 63);
          break;
        }
      }
    }
    free(buckets);
    free(next);
    free(member);
  }
  return 0;
}
