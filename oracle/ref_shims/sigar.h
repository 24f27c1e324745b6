/* Stand-in for the sigar system-information library, which the reference's
 * SystemUtils.cpp uses only to read the host's total and used memory.  It
 * reports a very large, empty memory so the reference never spills grids to
 * disk.  Test infrastructure for oracle/ref_harness.cpp only. */
#ifndef CAGEO_ORACLE_FAKE_SIGAR_H
#define CAGEO_ORACLE_FAKE_SIGAR_H
typedef struct { int unused; } sigar_t;
typedef struct { unsigned long long total, used, free, actual_used, actual_free, ram; double used_percent, free_percent; } sigar_mem_t;
#define SIGAR_OK 0
static inline int sigar_open(sigar_t** s) { static sigar_t one; *s = &one; return SIGAR_OK; }
static inline int sigar_close(sigar_t* s) { (void)s; return SIGAR_OK; }
static inline int sigar_mem_get(sigar_t* s, sigar_mem_t* m) {
  (void)s; m->total = 1ULL << 50; m->ram = 1ULL << 30; m->used = 0; m->free = m->total;
  m->actual_used = 0; m->actual_free = m->total; m->used_percent = 0; m->free_percent = 100; return SIGAR_OK; }
#endif
