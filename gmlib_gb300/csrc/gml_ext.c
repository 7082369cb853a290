/*
 * gml_ext.c -- extensions of the GB300 GMlib that have no counterpart in the
 * reference API: non-variadic forms for foreign-function callers, the offline
 * code-generation instance, launch controls, the NVRTC cubin cache, reductions
 * with indices, and the synthetic-mesh and Hilbert renumbering utilities.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>
#include <unistd.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"

/* ========================================================================= */
/* interned names                                                             */
/* ========================================================================= */

/* Link names built by GmlCompileKernel are kept for the life of the instance
   (the reference stores pointers to stack buffers, sources/gmlib3.c:2266-2283
   and :1053). */
const char *gmlx_intern(GmlSct *gml, const char *s)
{
   int i;
   for(i=0;i<gml->NmbNames;i++)
      if(!strcmp(gml->Names[i], s))
         return gml->Names[i];
   if(gml->NmbNames == gml->CapNames)
   {
      int cap = gml->CapNames ? 2 * gml->CapNames : 32;
      char **n = realloc(gml->Names, cap * sizeof(char *));
      if(!n)
         return s;
      gml->Names = n;
      gml->CapNames = cap;
   }
   gml->Names[ gml->NmbNames ] = strdup(s);
   return gml->Names[ gml->NmbNames++ ];
}

int gmlx_timing_off(GmlSct *gml)
{
   return gml->TimOff;
}

void gmlx_native_release(GmlSct *gml);
void gmlx_batch_release(GmlSct *gml);

void gmlx_release_extensions(GmlSct *gml)
{
   int i;
   gmlx_batch_release(gml);
   gmlx_native_release(gml);
   for(i=0;i<gml->NmbNames;i++)
      free(gml->Names[i]);
   free(gml->Names);
   gml->Names = NULL;
   gml->NmbNames = gml->CapNames = 0;
}

/* ========================================================================= */
/* cubin cache (process wide)                                                 */
/* ========================================================================= */

typedef struct CacheEnt
{
   uint64_t h;
   char *name;
   void *cubin;
   size_t size;
   struct CacheEnt *next;
}CacheEnt;

static CacheEnt *cache_head;
static pthread_mutex_t cache_lock = PTHREAD_MUTEX_INITIALIZER;

static uint64_t cache_key(const char *src, const char *opts)
{
   uint64_t h = gml_hash64(src, strlen(src), 0x5bd1e995ULL);
   return gml_hash64(opts ? opts : "", opts ? strlen(opts) : 0, h);
}

static int disk_path(char *buf, size_t n, uint64_t h, const char *name)
{
   const char *dir = getenv("GML_CACHE_DIR");
   if(!dir || !*dir)
      return 0;
   snprintf(buf, n, "%s/%016llx_%s.cubin", dir, (unsigned long long)h, name);
   return 1;
}

int gmlx_cache_lookup(const char *src, const char *opts, const char *name, void **cubin, size_t *size)
{
   uint64_t h = cache_key(src, opts);
   CacheEnt *e;
   char path[1024];
   FILE *f;

   pthread_mutex_lock(&cache_lock);
   for(e=cache_head;e;e=e->next)
      if(e->h == h && !strcmp(e->name, name))
      {
         *cubin = malloc(e->size);
         memcpy(*cubin, e->cubin, e->size);
         *size = e->size;
         pthread_mutex_unlock(&cache_lock);
         return 1;
      }
   pthread_mutex_unlock(&cache_lock);

   if(disk_path(path, sizeof(path), h, name) && (f = fopen(path, "rb")))
   {
      long n;
      fseek(f, 0, SEEK_END);
      n = ftell(f);
      fseek(f, 0, SEEK_SET);
      if(n > 0 && (*cubin = malloc(n)) && fread(*cubin, 1, n, f) == (size_t)n)
      {
         fclose(f);
         *size = n;
         gmlx_cache_store(src, opts, name, *cubin, *size);
         return 1;
      }
      fclose(f);
   }
   return 0;
}

void gmlx_cache_store(const char *src, const char *opts, const char *name, const void *cubin, size_t size)
{
   uint64_t h = cache_key(src, opts);
   CacheEnt *e = calloc(1, sizeof(CacheEnt));
   char path[1024];
   FILE *f;

   if(!e)
      return;
   e->h = h;
   e->name = strdup(name);
   e->cubin = malloc(size);
   memcpy(e->cubin, cubin, size);
   e->size = size;

   pthread_mutex_lock(&cache_lock);
   e->next = cache_head;
   cache_head = e;
   pthread_mutex_unlock(&cache_lock);

   if(disk_path(path, sizeof(path), h, name) && (f = fopen(path, "wb")))
   {
      fwrite(cubin, 1, size, f);
      fclose(f);
   }
}

/* ========================================================================= */
/* tuning table (process wide, kept in GML_CACHE_DIR/tune.json when set)      */
/* ========================================================================= */

/* Choices of the autotuners: the block size of a generated kernel, keyed by
   its source hash, the binary order of magnitude of its line count and the
   GPU's SM count ("k:<hash>:<log2 lines>:<sms>"), and the ball-of-points
   sorting window of a mesh ("w:<log2 vertices>:<sms>").  The file is a
   JSON object with one "key": value pair per line; it is read once and
   rewritten after every new choice. */
typedef struct TuneEnt
{
   char key[64];
   int val;
   struct TuneEnt *next;
}TuneEnt;

static TuneEnt *tune_head;
static int tune_loaded;
static pthread_mutex_t tune_lock = PTHREAD_MUTEX_INITIALIZER;

static int tune_path(char *buf, size_t n)
{
   const char *dir = getenv("GML_CACHE_DIR");
   if(!dir || !*dir)
      return 0;
   snprintf(buf, n, "%s/tune.json", dir);
   return 1;
}

static TuneEnt *tune_find(const char *key)
{
   for(TuneEnt *e=tune_head;e;e=e->next)
      if(!strcmp(e->key, key))
         return e;
   return NULL;
}

static void tune_put(const char *key, int val)
{
   TuneEnt *e = tune_find(key);
   if(!e && (e = calloc(1, sizeof(TuneEnt))))
   {
      snprintf(e->key, sizeof(e->key), "%s", key);
      e->next = tune_head;
      tune_head = e;
   }
   if(e)
      e->val = val;
}

static void tune_load(void)
{
   char path[1024], line[256], key[64];
   int val;
   FILE *f;
   if(tune_loaded)
      return;
   tune_loaded = 1;
   if(!tune_path(path, sizeof(path)) || !(f = fopen(path, "r")))
      return;
   while(fgets(line, sizeof(line), f))
      if(sscanf(line, " \"%63[^\"]\" : %d", key, &val) == 2)
         tune_put(key, val);
   fclose(f);
}

static void tune_save(void)
{
   char path[1024], tmp[1100];
   FILE *f;
   if(!tune_path(path, sizeof(path)))
      return;
   snprintf(tmp, sizeof(tmp), "%s.%d", path, (int)getpid());
   if(!(f = fopen(tmp, "w")))
      return;
   fprintf(f, "{\n");
   for(TuneEnt *e=tune_head;e;e=e->next)
      fprintf(f, "\"%s\": %d%s\n", e->key, e->val, e->next ? "," : "");
   fprintf(f, "}\n");
   if(fclose(f) == 0)
      rename(tmp, path);
   else
      remove(tmp);
}

static int log2_floor(long long n)
{
   int l = 0;
   while(n > 1) { n >>= 1; l++; }
   return l;
}

int gmlx_tune_get(const char *kind, uint64_t hash, long long count, int nsm)
{
   char key[64];
   TuneEnt *e;
   int val = 0;
   snprintf(key, sizeof(key), "%s:%016llx:%d:%d", kind, (unsigned long long)hash,
            log2_floor(count), nsm);
   pthread_mutex_lock(&tune_lock);
   tune_load();
   if((e = tune_find(key)))
      val = e->val;
   pthread_mutex_unlock(&tune_lock);
   return val;
}

void gmlx_tune_set(const char *kind, uint64_t hash, long long count, int nsm, int val)
{
   char key[64];
   snprintf(key, sizeof(key), "%s:%016llx:%d:%d", kind, (unsigned long long)hash,
            log2_floor(count), nsm);
   pthread_mutex_lock(&tune_lock);
   tune_load();
   tune_put(key, val);
   tune_save();
   pthread_mutex_unlock(&tune_lock);
}

/* ========================================================================= */
/* instance control                                                           */
/* ========================================================================= */

size_t GmlxInitOffline(void)
{
   GmlSct *gml = calloc(1, sizeof(GmlSct));
   if(!gml)
      return 0;
   gml->Offline = 1;
   gml->dev = NULL;
   gml->DblExt = 1;
   gml->RedScrSiz = gmd_reduce_scratch_bytes(0);
   gml->RedScr = gmd_alloc(NULL, gml->RedScrSiz);
   gml->TimOff = 1;
   return (size_t)gml;
}

int GmlxSetTiming(size_t GmlIdx, int on)
{
   GETGMLPTR(gml, GmlIdx);
   gml->TimOff = on ? 0 : 1;
   return 1;
}

int GmlxSetTuning(size_t GmlIdx, int on, int block)
{
   GETGMLPTR(gml, GmlIdx);
   int i;
   gml->TunOff = on ? 0 : 1;
   gml->TunBlk = block > 0 ? block : 256;
   if(!on)
      for(i=1;i<=gml->NmbKrn && i<=GmlMaxKrn;i++)
         if(gml->krn[i].kind == GmlKrnGenerated)
         {
            int lim = gml->krn[i].MaxSiz > 0 ? gml->krn[i].MaxSiz : 1024;
            gml->krn[i].OptSiz = gml->TunBlk < lim ? gml->TunBlk : lim;
         }
   return 1;
}

static GmlKrnSct *get_krn(GmlSct *gml, int idx)
{
   if(idx < 1 || idx > gml->NmbKrn || idx > GmlMaxKrn || !gml->krn[idx].use)
      return NULL;
   return &gml->krn[idx];
}

int GmlxKernelBlockSize(size_t GmlIdx, int KrnIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *k = get_krn(gml, KrnIdx);
   return k ? k->OptSiz : -1;
}

const char *GmlxKernelSource(size_t GmlIdx, int KrnIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *k = get_krn(gml, KrnIdx);
   return k ? k->source : NULL;
}

int GmlxKernelIsLazy(size_t GmlIdx, int KrnIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *k = get_krn(gml, KrnIdx);
   return k ? k->lazy : -1;
}

int GmlxKernelRegisters(size_t GmlIdx, int KrnIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *k = get_krn(gml, KrnIdx);
   return k ? k->NumReg : -1;
}

int GmlxSetLazy(size_t GmlIdx, int on)
{
   GETGMLPTR(gml, GmlIdx);
   gml->LazyOff = on ? 0 : 1;
   return 1;
}

int GmlxLinkData(size_t GmlIdx, int SrcTyp, int DstTyp, int *BalIdx, int *DegIdx, int *HghIdx)
{
   GETGMLPTR(gml, GmlIdx);
   if(SrcTyp < 0 || SrcTyp >= GmlMaxEleTyp || DstTyp < 0 || DstTyp >= GmlMaxEleTyp)
      return 0;
   if(BalIdx) *BalIdx = gml->LnkMat[ SrcTyp ][ DstTyp ];
   if(DegIdx) *DegIdx = gml->CntMat[ SrcTyp ][ DstTyp ];
   if(HghIdx) *HghIdx = gml->LnkHgh[ SrcTyp ][ DstTyp ];
   return gml->LnkMat[ SrcTyp ][ DstTyp ] ? 1 : 0;
}

int GmlxSynchronize(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   return gmd_sync(gml->dev);
}

void *GmlxStream(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   return gmd_stream(gml->dev);
}

void *GmlxEventCreate(void)              { return gmd_event_new(); }
int GmlxEventRecord(size_t GmlIdx, void *evt)
{
   GETGMLPTR(gml, GmlIdx);
   return gmd_event_record(gml->dev, evt);
}
double GmlxEventElapsed(void *beg, void *end) { return gmd_event_elapsed_s(beg, end); }
void GmlxEventDestroy(void *evt)         { gmd_event_free(evt); }

/* ========================================================================= */
/* non-variadic forms                                                         */
/* ========================================================================= */

int GmlxCompileKernelV(size_t GmlIdx, const char *src, const char *name, int MshTyp,
                       int NmbTyp, const int *IdxTab, const int *FlgTab, const int *LnkTab)
{
   int t[3 * 8];
   if(NmbTyp < 1 || NmbTyp > 8)
   {
      printf("GmlxCompileKernelV: 1 to 8 datatypes are supported\n");
      return 0;
   }
   for(int i=0;i<8;i++)
   {
      t[3*i]   = i < NmbTyp ? IdxTab[i] : 0;
      t[3*i+1] = i < NmbTyp ? FlgTab[i] : 0;
      t[3*i+2] = i < NmbTyp && LnkTab ? LnkTab[i] : 0;
   }
   return GmlCompileKernel(GmlIdx, (char *)src, (char *)name, MshTyp, NmbTyp,
                           t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8],
                           t[9], t[10], t[11], t[12], t[13], t[14], t[15], t[16], t[17],
                           t[18], t[19], t[20], t[21], t[22], t[23]);
}

static GmlDatSct *get_dat(GmlSct *gml, int idx)
{
   if(idx < 1 || idx > GmlMaxDat || !gml->dat[idx].use)
      return NULL;
   return &gml->dat[idx];
}

/* Whole-datatype transfers.  Staged path (as GmlSetDataBlock /
   GmlGetDataBlock): the caller's buffer is copied into the pinned host
   mirror on the CPU, and the mirror is uploaded or downloaded by DMA.  On
   this platform one CPU thread copies about 15 GB/s, against about 200 GB/s
   for the chip-to-chip link, so the host copy is most of the time.  Direct
   path, taken for large pinned-mirror datatypes when the device can address
   the caller's buffer (gmd_host_addressable) and the instance is idle: one
   kernel reads the source once and writes both the destination and the
   mirror, so the mirror ends up exactly as on the staged path. */
#define GML_DIRECT_MIN (1u << 20)

static int direct_ok(GmlSct *gml, GmlDatSct *dat, const void *buf, size_t bytes)
{
   return bytes >= GML_DIRECT_MIN && dat->pinned && dat->GpuMem
       && gmd_host_addressable(gml->dev, buf);
}

/* A datatype's mirror is rewritten whole: a refresh still owed to it is
   dropped (it would be overwritten), the ones owed to other datatypes wait
   (their device data do not change here). */
static void drop_refresh(GmlSct *gml, GmlDatSct *dat)
{
   if(dat->MirOld)
   {
      dat->MirOld = 0;
      gml->NmbMirOld--;
   }
}

int GmlxSetData(size_t GmlIdx, int DatIdx, const void *buf, size_t bytes)
{
   GETGMLPTR_NOSETTLE(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   if(!dat || !dat->CpuMem || bytes != dat->MemSiz)
   {
      gml_settle(gml);
      return 0;
   }
   drop_refresh(gml, dat);
   gml_wait_upload(gml, dat);
   if(gml->MirOff)
   {
      /* an instance whose mirrors nobody reads: the device copy only, with
         one kernel when the device can address buf, else by DMA */
      if(!(gmd_host_addressable(gml->dev, buf) && gmd_fanout(gml->dev, buf, dat->GpuMem, NULL, bytes))
      && !gmd_h2d_async(gml->dev, dat->GpuMem, buf, bytes))
         return 0;
      if(!gmd_sync(gml->dev))
         return 0;
      gml->MovSiz += bytes;
      return 1;
   }
   /* direct only when idle: the copy must land before the call returns (the
      caller may reuse buf), and waiting behind queued kernels would make an
      asynchronous upload blocking */
   if(dat->MemAcs != GmlOutput && direct_ok(gml, dat, buf, bytes) && gmd_idle(gml->dev)
   && gmd_fanout(gml->dev, buf, dat->GpuMem, dat->CpuMem, bytes))
   {
      if(!gmd_sync(gml->dev))
         return 0;
      gml->MovSiz += bytes;
      return 1;
   }
   gml_host_copy(dat->CpuMem, buf, bytes);
   return gml_upload(gml, DatIdx) || !bytes;
}

int GmlxGetData(size_t GmlIdx, int DatIdx, void *buf, size_t bytes)
{
   GETGMLPTR_NOSETTLE(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   if(!dat || !dat->CpuMem || bytes != dat->MemSiz)
   {
      gml_settle(gml);
      return 0;
   }
   if(direct_ok(gml, dat, buf, bytes))
   {
      /* ordered after the kernels that produced the data; the mirror is
         refreshed at the next call on the instance (gml_settle), where a
         download would have refreshed it here: until then nothing can
         read it or change the device data.  Reads of other datatypes whose
         refresh is owed leave theirs owed too. */
      gml_wait_upload(gml, dat);
      if(gmd_fanout(gml->dev, dat->GpuMem, buf, NULL, bytes))
      {
         if(!gmd_sync(gml->dev))
            return 0;
         if(!dat->MirOld)
         {
            dat->MirOld = 1;
            gml->NmbMirOld++;
         }
         gml->MovSiz += bytes;
         return 1;
      }
   }
   drop_refresh(gml, dat);
   if(!gml_download(gml, DatIdx) && bytes)
      return 0;
   gml_host_copy(buf, dat->CpuMem, bytes);
   return 1;
}

size_t GmlxDataBytes(size_t GmlIdx, int DatIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   return dat ? dat->MemSiz : 0;
}

int GmlxDataLines(size_t GmlIdx, int DatIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   return dat ? dat->NmbLin : -1;
}

void *GmlxDevicePtr(size_t GmlIdx, int DatIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   return dat ? dat->GpuMem : NULL;
}

int GmlxReduceArg(size_t GmlIdx, int DatIdx, float *MinVal, int *MinIdx, float *MaxVal, int *MaxIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = get_dat(gml, DatIdx);
   if(!dat || dat->ItmTyp != GmlFlt || dat->NmbItm != 1 || dat->NmbLin < 1)
      return 0;
   if(gml->Offline)
      return 0;
   return gmd_minmax_arg_f32(gml->dev, (const float *)dat->GpuMem, dat->NmbLin,
                             MinVal, MinIdx, MaxVal, MaxIdx, gml->RedScr);
}

/* ========================================================================= */
/* synthetic cube meshes                                                      */
/* ========================================================================= */

void GmlxCubeSizes(int n, int *NmbVer, int *NmbTet)
{
   if(NmbVer) *NmbVer = (n + 1) * (n + 1) * (n + 1);
   if(NmbTet) *NmbTet = 6 * n * n * n;
}

static uint64_t splitmix64(uint64_t *s)
{
   uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
   z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
   z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
   return z ^ (z >> 31);
}

/* uniform double in [-1, 1) from 53 random bits */
static double unit_sym(uint64_t *s)
{
   return ((double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

int GmlxCubeMesh(int n, int split, double jitter, uint64_t seed, float *crd, int *tet, int *ref)
{
   int i, j, k, p, m = n + 1;
   double h = 1.0 / n;
   /* the 6 permutations of the axes: paths from a corner to its opposite */
   static const int perm[6][3] = { {0,1,2}, {0,2,1}, {1,0,2}, {1,2,0}, {2,0,1}, {2,1,0} };

   if(n < 1)
      return 0;

   for(k=0;k<m;k++)
      for(j=0;j<m;j++)
         for(i=0;i<m;i++)
         {
            size_t v = (size_t)i + (size_t)m * ((size_t)j + (size_t)m * k);
            int bnd = (i == 0 || j == 0 || k == 0 || i == n || j == n || k == n);
            double x = i * h, y = j * h, z = k * h;
            if(!bnd && jitter != 0.)
            {
               uint64_t s = seed ^ (0xd1b54a32d192ed03ULL * (uint64_t)(v + 1));
               x += unit_sym(&s) * jitter * h;
               y += unit_sym(&s) * jitter * h;
               z += unit_sym(&s) * jitter * h;
            }
            crd[ 4*v ] = (float)x;
            crd[ 4*v+1 ] = (float)y;
            crd[ 4*v+2 ] = (float)z;
            crd[ 4*v+3 ] = 0.f;
            if(ref)
               ref[v] = bnd;
         }

   for(k=0;k<n;k++)
      for(j=0;j<n;j++)
         for(i=0;i<n;i++)
         {
            size_t hex = (size_t)i + (size_t)n * ((size_t)j + (size_t)n * k);
            int s0 = split ? ((i & 1) | ((j & 1) << 1) | ((k & 1) << 2)) : 0;
            for(p=0;p<6;p++)
            {
               int c[4], q, cur = s0, v[4];
               c[0] = cur;
               for(q=0;q<3;q++)
               {
                  cur ^= 1 << perm[p][q];
                  c[q+1] = cur;
               }
               for(q=0;q<4;q++)
               {
                  int dx = c[q] & 1, dy = (c[q] >> 1) & 1, dz = (c[q] >> 2) & 1;
                  v[q] = (i + dx) + m * ((j + dy) + m * (k + dz));
               }
               /* positive orientation on the undeformed cube: the sign of a
                  path tet follows the parity of its corner sequence */
               {
                  int a[3][3], d, t;
                  for(q=0;q<3;q++)
                  {
                     a[q][0] = ((c[q+1] & 1) - (c[0] & 1));
                     a[q][1] = (((c[q+1] >> 1) & 1) - ((c[0] >> 1) & 1));
                     a[q][2] = (((c[q+1] >> 2) & 1) - ((c[0] >> 2) & 1));
                  }
                  d = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1])
                    - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0])
                    + a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
                  if(d < 0)
                  {
                     t = v[2]; v[2] = v[3]; v[3] = t;
                  }
               }
               for(q=0;q<4;q++)
                  tet[ 4 * (6 * hex + p) + q ] = v[q];
            }
         }

   return 1;
}

/* ========================================================================= */
/* Hilbert renumbering                                                        */
/* ========================================================================= */

/* Hilbert index of a point with 21-bit integer coordinates, following
   J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707 (2004):
   axes to transpose form, then bit interleaving. */
static uint64_t hilbert_key(uint32_t x0, uint32_t x1, uint32_t x2)
{
   uint32_t X[3] = { x0, x1, x2 }, M = 1u << 20, P, Q, t;
   int i;
   uint64_t key = 0;

   for(Q=M;Q>1;Q>>=1)
   {
      P = Q - 1;
      for(i=0;i<3;i++)
      {
         if(X[i] & Q)
            X[0] ^= P;
         else
         {
            t = (X[0] ^ X[i]) & P;
            X[0] ^= t;
            X[i] ^= t;
         }
      }
   }
   for(i=1;i<3;i++)
      X[i] ^= X[i-1];
   t = 0;
   for(Q=M;Q>1;Q>>=1)
      if(X[2] & Q)
         t ^= Q - 1;
   for(i=0;i<3;i++)
      X[i] ^= t;

   for(int b=20;b>=0;b--)
      for(i=0;i<3;i++)
         key = (key << 1) | ((X[i] >> b) & 1);
   return key;
}

typedef struct { uint64_t key; int idx; } KeyIdx;

static int cmp_keyidx(const void *a, const void *b)
{
   const KeyIdx *x = a, *y = b;
   if(x->key != y->key) return x->key < y->key ? -1 : 1;
   return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

int GmlxHilbertRenumber(int NmbVer, float *crd, int *ref, int NmbTet, int *tet, int *VerPrm)
{
   float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
   double sc[3];
   KeyIdx *ki;
   int *nw, i, d, *tmpi;
   float *tmpf;

   if(NmbVer < 1)
      return 0;

   for(i=0;i<NmbVer;i++)
      for(d=0;d<3;d++)
      {
         if(crd[4*i+d] < lo[d]) lo[d] = crd[4*i+d];
         if(crd[4*i+d] > hi[d]) hi[d] = crd[4*i+d];
      }
   for(d=0;d<3;d++)
      sc[d] = hi[d] > lo[d] ? 2097151.0 / ((double)hi[d] - lo[d]) : 0.;

   ki = malloc((size_t)(NmbVer > NmbTet ? NmbVer : NmbTet) * sizeof(KeyIdx));
   nw = malloc((size_t)NmbVer * sizeof(int));
   if(!ki || !nw) { free(ki); free(nw); return 0; }

   for(i=0;i<NmbVer;i++)
   {
      uint32_t q[3];
      for(d=0;d<3;d++)
         q[d] = (uint32_t)(((double)crd[4*i+d] - lo[d]) * sc[d]);
      ki[i].key = hilbert_key(q[0], q[1], q[2]);
      ki[i].idx = i;
   }
   qsort(ki, NmbVer, sizeof(KeyIdx), cmp_keyidx);
   for(i=0;i<NmbVer;i++)
      nw[ ki[i].idx ] = i;

   tmpf = malloc((size_t)NmbVer * 4 * sizeof(float));
   tmpi = malloc((size_t)NmbVer * sizeof(int));
   if(!tmpf || !tmpi) { free(ki); free(nw); free(tmpf); free(tmpi); return 0; }
   for(i=0;i<NmbVer;i++)
   {
      memcpy(&tmpf[ 4 * nw[i] ], &crd[ 4*i ], 4 * sizeof(float));
      if(ref) tmpi[ nw[i] ] = ref[i];
   }
   memcpy(crd, tmpf, (size_t)NmbVer * 4 * sizeof(float));
   if(ref) memcpy(ref, tmpi, (size_t)NmbVer * sizeof(int));
   free(tmpf);
   free(tmpi);

   if(NmbTet > 0 && tet)
   {
      int *tt = malloc((size_t)NmbTet * 4 * sizeof(int));
      if(!tt) { free(ki); free(nw); return 0; }
      for(i=0;i<NmbTet*4;i++)
         tet[i] = nw[ tet[i] ];
      for(i=0;i<NmbTet;i++)
      {
         double c[3] = { 0, 0, 0 };
         uint32_t q[3];
         for(int v=0;v<4;v++)
            for(d=0;d<3;d++)
               c[d] += 0.25 * crd[ 4 * tet[4*i+v] + d ];
         for(d=0;d<3;d++)
            q[d] = (uint32_t)((c[d] - lo[d]) * sc[d]);
         ki[i].key = hilbert_key(q[0], q[1], q[2]);
         ki[i].idx = i;
      }
      qsort(ki, NmbTet, sizeof(KeyIdx), cmp_keyidx);
      for(i=0;i<NmbTet;i++)
         memcpy(&tt[ 4*i ], &tet[ 4 * ki[i].idx ], 4 * sizeof(int));
      memcpy(tet, tt, (size_t)NmbTet * 4 * sizeof(int));
      free(tt);
   }

   if(VerPrm)
      memcpy(VerPrm, nw, (size_t)NmbVer * sizeof(int));

   free(ki);
   free(nw);
   return 1;
}

/* Stable partition of the vertices by tetrahedron degree, the second half
   of the reference's renumbering (lower degrees first, higher degrees at
   the end of the table, Documentation/GMlib3_en.tex:401): vertices in at
   most BalSiz tetrahedra first, then the others, each group in its previous
   order.  The ball tables start their wide part at the first vertex above
   BalSiz (gmlib3.c:930-937), so without this every vertex behind that one
   goes through the wide table. */
int GmlxDegreeSort(int NmbVer, float *crd, int *ref, int NmbTet, int *tet, int BalSiz,
                   int *VerPrm)
{
   int *deg, *nw, *tmpi, i, low = 0, pos[2];
   float *tmpf;

   if(NmbVer < 1 || NmbTet < 0 || (NmbTet > 0 && !tet) || !crd || BalSiz < 1)
      return -1;
   deg = calloc((size_t)NmbVer, sizeof(int));
   nw = malloc((size_t)NmbVer * sizeof(int));
   tmpf = malloc((size_t)NmbVer * 4 * sizeof(float));
   tmpi = malloc((size_t)NmbVer * sizeof(int));
   if(!deg || !nw || !tmpf || !tmpi)
   {
      free(deg); free(nw); free(tmpf); free(tmpi);
      return -1;
   }
   for(i=0;i<4*NmbTet;i++)
   {
      if(tet[i] < 0 || tet[i] >= NmbVer)
      {
         free(deg); free(nw); free(tmpf); free(tmpi);
         return -1;
      }
      deg[ tet[i] ]++;
   }
   for(i=0;i<NmbVer;i++)
      low += deg[i] <= BalSiz;
   pos[0] = 0;
   pos[1] = low;
   for(i=0;i<NmbVer;i++)
      nw[i] = pos[ deg[i] > BalSiz ]++;

   for(i=0;i<NmbVer;i++)
   {
      memcpy(&tmpf[ 4 * nw[i] ], &crd[ 4*i ], 4 * sizeof(float));
      if(ref) tmpi[ nw[i] ] = ref[i];
   }
   memcpy(crd, tmpf, (size_t)NmbVer * 4 * sizeof(float));
   if(ref) memcpy(ref, tmpi, (size_t)NmbVer * sizeof(int));
   for(i=0;i<4*NmbTet;i++)
      tet[i] = nw[ tet[i] ];
   if(VerPrm)
      memcpy(VerPrm, nw, (size_t)NmbVer * sizeof(int));

   free(deg); free(nw); free(tmpf); free(tmpi);
   return low;
}
