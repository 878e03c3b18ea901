/*
 * Test infrastructure only: a pthread stand-in for the four binary-only
 * runtime libraries the reference links (Spindle, Parutil, Silo, Topo), so the
 * reference's own C sources can be compiled and run here as the oracle
 * (`oracle/_ref/wedge_ref`).  Nothing in the product links this file.
 *
 * Each function restates the behaviour documented in the reference's headers:
 *   third_party/include/spindle.h:72-158  (SPMD threads, IDs, barriers)
 *   third_party/include/parutil.h:138-203 (chunked static schedule, memset)
 *   third_party/include/silo.h:41-76      (NUMA buffers -> plain aligned heap)
 * The reference is always run here with one task (one NUMA node), so local and
 * global IDs/barriers coincide.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <parutil.h>
#include <silo.h>
#include <spindle.h>

/* thread count used when a task spec asks for "all available" threads */
uint32_t shim_default_threads = 1;

typedef struct {
    uint32_t local_id, global_id, task_id, local_count, global_count, task_count;
    bool in_region;
} shim_tls_t;

static __thread shim_tls_t tls;

static pthread_barrier_t barrier_global;
static pthread_barrier_t barrier_task[8];

typedef struct {
    TSpindleFunc func;
    void* arg;
    shim_tls_t ids;
} shim_start_t;

static void* shim_thread_main(void* p)
{
    shim_start_t* s = (shim_start_t*)p;
    tls = s->ids;
    tls.in_region = true;
    s->func(s->arg);
    tls.in_region = false;
    return NULL;
}

uint32_t spindleThreadsSpawn(SSpindleTaskSpec* taskSpec, uint32_t taskCount, bool useCurrentThread)
{
    uint32_t counts[8];
    uint32_t total = 0;
    if (taskCount == 0 || taskCount > 8)
        return 1;
    for (uint32_t t = 0; t < taskCount; ++t) {
        counts[t] = taskSpec[t].numThreads == 0 ? shim_default_threads : taskSpec[t].numThreads;
        total += counts[t];
    }
    pthread_barrier_init(&barrier_global, NULL, total);
    for (uint32_t t = 0; t < taskCount; ++t)
        pthread_barrier_init(&barrier_task[t], NULL, counts[t]);

    shim_start_t* starts = (shim_start_t*)calloc(total, sizeof(shim_start_t));
    pthread_t* th = (pthread_t*)calloc(total, sizeof(pthread_t));
    uint32_t g = 0;
    for (uint32_t t = 0; t < taskCount; ++t) {
        for (uint32_t l = 0; l < counts[t]; ++l, ++g) {
            starts[g].func = taskSpec[t].func;
            starts[g].arg = taskSpec[t].arg;
            starts[g].ids.local_id = l;
            starts[g].ids.global_id = g;
            starts[g].ids.task_id = t;
            starts[g].ids.local_count = counts[t];
            starts[g].ids.global_count = total;
            starts[g].ids.task_count = taskCount;
        }
    }
    shim_tls_t saved = tls;
    for (uint32_t i = (useCurrentThread ? 1u : 0u); i < total; ++i)
        pthread_create(&th[i], NULL, shim_thread_main, &starts[i]);
    if (useCurrentThread)
        shim_thread_main(&starts[0]);
    for (uint32_t i = (useCurrentThread ? 1u : 0u); i < total; ++i)
        pthread_join(th[i], NULL);
    tls = saved;
    pthread_barrier_destroy(&barrier_global);
    for (uint32_t t = 0; t < taskCount; ++t)
        pthread_barrier_destroy(&barrier_task[t]);
    free(starts);
    free(th);
    return 0;
}

bool spindleIsInParallelRegion(void) { return tls.in_region; }
uint32_t spindleGetLocalThreadID(void) { return tls.local_id; }
uint32_t spindleGetGlobalThreadID(void) { return tls.global_id; }
uint32_t spindleGetTaskID(void) { return tls.task_id; }
uint32_t spindleGetLocalThreadCount(void) { return tls.local_count; }
uint32_t spindleGetGlobalThreadCount(void) { return tls.global_count; }
uint32_t spindleGetTaskCount(void) { return tls.task_count; }
void spindleBarrierLocal(void) { pthread_barrier_wait(&barrier_task[tls.task_id]); }
void spindleBarrierGlobal(void) { pthread_barrier_wait(&barrier_global); }

bool parutilSchedulerStatic(const EParutilStaticScheduler type, const uint64_t units, SParutilStaticSchedule* const schedule)
{
    (void)type;
    if (schedule == NULL)
        return false;
    const uint64_t n = tls.in_region ? tls.local_count : 1;
    const uint64_t id = tls.in_region ? tls.local_id : 0;
    const uint64_t per = units / n, extra = units % n;
    schedule->startUnit = per * id + (id < extra ? id : extra);
    schedule->endUnit = schedule->startUnit + per + (id < extra ? 1 : 0);
    schedule->increment = 1;
    return true;
}

void* parutilMemorySet(void* buffer, uint8_t value, size_t num)
{
    if (!tls.in_region) {
        memset(buffer, value, num);
        return buffer;
    }
    const uint64_t n = tls.local_count, id = tls.local_id;
    const uint64_t per = num / n, extra = num % n;
    const uint64_t start = per * id + (id < extra ? id : extra);
    const uint64_t len = per + (id < extra ? 1 : 0);
    memset((uint8_t*)buffer + start, value, len);
    pthread_barrier_wait(&barrier_task[tls.task_id]);
    return buffer;
}

void* siloSimpleBufferAlloc(size_t size, uint32_t numaNode)
{
    (void)numaNode;
    void* p = NULL;
    size_t rounded = (size + 4095) & ~(size_t)4095;
    if (rounded == 0)
        rounded = 4096;
    if (posix_memalign(&p, 4096, rounded) != 0)
        return NULL;
    return p;
}

void* siloMultinodeArrayAlloc(uint32_t count, const SSiloMemorySpec* spec)
{
    size_t total = 0;
    for (uint32_t i = 0; i < count; ++i)
        total += (spec[i].size + 4095) & ~(size_t)4095;
    return siloSimpleBufferAlloc(total, 0);
}

void siloFree(void* ptr) { free(ptr); }
