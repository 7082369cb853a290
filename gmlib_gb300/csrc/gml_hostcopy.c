/*
 * gml_hostcopy.c -- host memory copies between caller buffers and the
 * pinned host mirrors of datatypes.
 *
 * A single thread copies about 10-20 GB/s on the host, well below what the
 * CPU-GPU link moves, so whole-datatype transfers (GmlxSetData /
 * GmlxGetData) would be bound by that memcpy.  Copies of 8 MB and more are
 * split over up to 8 threads (the calling thread takes one share).  Only
 * one such split copy runs at a time in the process: callers that copy from
 * several threads at once (the request loop) would otherwise oversubscribe
 * the cores, so a copy that finds another one running stays single-threaded.
 */
#include <pthread.h>
#include <string.h>
#include "gml_internal.h"

#define HC_MIN_BYTES  (8u << 20)
#define HC_MAX_THREADS 8

typedef struct
{
   char        *dst;
   const char  *src;
   size_t      n;
}HcJob;

static void *hc_run(void *arg)
{
   HcJob *j = (HcJob *)arg;
   memcpy(j->dst, j->src, j->n);
   return NULL;
}

static int hc_busy;

void gml_host_copy(void *dst, const void *src, size_t n)
{
   HcJob job[HC_MAX_THREADS];
   pthread_t th[HC_MAX_THREADS];
   int started[HC_MAX_THREADS] = { 0 };
   size_t share, off = 0;
   int nt = 1, i;

   if(n >= HC_MIN_BYTES && !__atomic_exchange_n(&hc_busy, 1, __ATOMIC_ACQUIRE))
      nt = HC_MAX_THREADS;
   else
   {
      memcpy(dst, src, n);
      return;
   }
   share = ((n / nt) + 4095) & ~(size_t)4095;
   for(i=0;i<nt;i++)
   {
      size_t len = off >= n ? 0 : (n - off < share ? n - off : share);
      job[i].dst = (char *)dst + off;
      job[i].src = (const char *)src + off;
      job[i].n = len;
      off += len;
   }
   /* threads 1..nt-1 in the background; a thread that cannot start is
      copied by the caller */
   for(i=1;i<nt;i++)
      if(job[i].n && pthread_create(&th[i], NULL, hc_run, &job[i]) == 0)
         started[i] = 1;
   hc_run(&job[0]);
   for(i=1;i<nt;i++)
   {
      if(started[i])
         pthread_join(th[i], NULL);
      else if(job[i].n)
         hc_run(&job[i]);
   }
   __atomic_store_n(&hc_busy, 0, __ATOMIC_RELEASE);
}
