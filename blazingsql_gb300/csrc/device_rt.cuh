// device_rt.cuh -- device-side runtime included (as text) ahead of every
// plan kernel the library JIT-compiles with NVRTC for sm_103a.
//
// Value model: every intermediate is 64 bits that an op reads as int64 or as
// double depending on its operand's kernel type, plus a validity bit -- the
// slot model of engine/src/Interpreter/interpreter_ops.cuh:248-262, kept in
// registers instead of a shared-memory slot file.  Plans are compiled with
// --fmad=false so every FP64 op rounds once, in the reference's op order.

typedef unsigned long long u64;
typedef long long i64;
typedef unsigned int u32;

#define GX_MAGIC_I 9223372036854775794LL   /* INT64_MAX - 13, interpreter_ops.cuh:41 */
#define GX_MAGIC_D 1.7976931348623123e+308 /* interpreter_ops.cuh:47 */
#define GX_FULL 0xffffffffu

// ---- bit views -------------------------------------------------------------
__device__ __forceinline__ double gx_D(u64 b) { return __longlong_as_double((i64)b); }
__device__ __forceinline__ u64 gx_B(double d) { return (u64)__double_as_longlong(d); }
__device__ __forceinline__ double gx_I2D(u64 b) { return (double)(i64)b; }
// static_cast<int64_t>(double) on the GPU: truncate, saturate, NaN -> 0
__device__ __forceinline__ i64 gx_D2LL(double d) { return __double2ll_rz(d); }

// ---- integer division guards (the reference's DIV marks /0 NULL) -----------
__device__ __forceinline__ u64 gx_div_ii(u64 a, u64 b) {
  const i64 x = (i64)a, y = (i64)b;
  return y == 0 ? 0ull : (y == -1 ? 0ull - a : (u64)(x / y));
}
__device__ __forceinline__ u64 gx_mod_ii(u64 a, u64 b) {
  const i64 x = (i64)a, y = (i64)b;
  return (y == 0 || y == -1) ? 0ull : (u64)(x % y);
}

// ---- ROUND scale: correctly rounded 10^d for integral |d| <= 22 -------------
__constant__ double gx_p10[23] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11,
                                  1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
__constant__ double gx_n10[23] = {1e-0, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11,
                                  1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17, 1e-18, 1e-19, 1e-20, 1e-21, 1e-22};
__device__ __forceinline__ double gx_pow10(double d) {
  if (d == floor(d) && d >= -22.0 && d <= 22.0) {
    const int k = (int)d;
    return k >= 0 ? gx_p10[k] : gx_n10[-k];
  }
  return pow(10.0, d);
}
__device__ __forceinline__ double gx_round_to(double x, double digits) {
  const double f = gx_pow10(digits);
  const double p = x * f;
  return round(p) / f;
}

// ---- timestamps ------------------------------------------------------------
// count of a timestamp/duration value: int32 representation for *_DAYS
__device__ __forceinline__ i64 gx_days32(i64 v) { return (i64)(int)v; }
__device__ __forceinline__ i64 gx_floordiv(i64 a, i64 b) {
  i64 q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
  return q;
}
// civil_from_days (H. Hinnant's published algorithm); part: 0 year, 1 month, 2 day
__device__ __forceinline__ i64 gx_civil(i64 days, int part) {
  const i64 z = days + 719468;
  const i64 era = (z >= 0 ? z : z - 146096) / 146097;
  const i64 doe = z - era * 146097;
  const i64 yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  const i64 doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const i64 mp = (5 * doy + 2) / 153;
  const i64 d = doy - (153 * mp + 2) / 5 + 1;
  const i64 m = mp < 10 ? mp + 3 : mp - 9;
  const i64 y = yoe + era * 400 + (m <= 2);
  return part == 0 ? y : (part == 1 ? m : d);
}
// EXTRACT on a timestamp count with `per_day` units per day (1 for DAYS).
// which: 0 year, 1 month, 2 day, 3 iso day-of-week, 4 hour, 5 minute, 6 second
__device__ __forceinline__ i64 gx_extract(i64 cnt, i64 per_day, int which) {
  const i64 days = per_day == 1 ? cnt : gx_floordiv(cnt, per_day);
  if (which <= 2) return gx_civil(days, which);
  if (which == 3) {
    const i64 wd = ((days % 7) + 7 + 4) % 7;
    return wd == 0 ? 7 : wd;
  }
  if (per_day == 1) return 0;
  const i64 tsm = cnt - days * per_day;
  const i64 ph = per_day / 24, pm = ph / 60, ps = pm / 60;
  if (which == 4) return tsm / ph;
  if (which == 5) return (tsm % ph) / pm;
  return (tsm % pm) / ps;
}

// ---- RAND: Philox4x32-10 (Salmon et al., SC'11) -> uniform double in (0, 1] -
__device__ __forceinline__ double gx_philox_uniform(u64 seed, u32 rand_id, u64 row) {
  u32 c0 = (u32)row, c1 = (u32)(row >> 32), c2 = rand_id, c3 = 0x5EEDu;
  u32 k0 = (u32)seed, k1 = (u32)(seed >> 32);
#pragma unroll
  for (int i = 0; i < 10; i++) {
    const u32 h0 = __umulhi(0xD2511F53u, c0), l0 = 0xD2511F53u * c0;
    const u32 h1 = __umulhi(0xCD9E8D57u, c2), l1 = 0xCD9E8D57u * c2;
    const u32 n0 = h1 ^ c1 ^ k0, n1 = l1, n2 = h0 ^ c3 ^ k1, n3 = l0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  const u64 m = ((u64)c0 << 21) | (c1 >> 11);
  return (double)(m + 1ull) * (1.0 / 9007199254740992.0);
}

// ---- validity --------------------------------------------------------------
__device__ __forceinline__ bool gx_valid(const u32* __restrict__ m, i64 bit) {
  return m == nullptr ? true : ((__ldg(m + (bit >> 5)) >> (bit & 31)) & 1u);
}

// ---- streaming loads / stores ------------------------------------------------
__device__ __forceinline__ i64 gx_ld_i8(const void* p, i64 i) { return (i64)__ldcs((const signed char*)p + i); }
__device__ __forceinline__ i64 gx_ld_u8(const void* p, i64 i) { return (i64)__ldcs((const unsigned char*)p + i); }
__device__ __forceinline__ i64 gx_ld_i16(const void* p, i64 i) { return (i64)__ldcs((const short*)p + i); }
__device__ __forceinline__ i64 gx_ld_u16(const void* p, i64 i) { return (i64)__ldcs((const unsigned short*)p + i); }
__device__ __forceinline__ i64 gx_ld_i32(const void* p, i64 i) { return (i64)__ldcs((const int*)p + i); }
__device__ __forceinline__ i64 gx_ld_u32(const void* p, i64 i) { return (i64)__ldcs((const unsigned int*)p + i); }
__device__ __forceinline__ u64 gx_ld_64(const void* p, i64 i) { return (u64)__ldcs((const long long*)p + i); }
__device__ __forceinline__ u64 gx_ld_f32(const void* p, i64 i) { return gx_B((double)__ldcs((const float*)p + i)); }
__device__ __forceinline__ u64 gx_ld_f32e(const void* p, i64 i) { return gxe_f2d(__ldcs((const unsigned*)p + i)); }

// the same loads with the default cache policy, for a column the predicate
// reads and the projections read again by kept row: its lines stay in L2
// between the two (a streaming load marks them first to evict)
__device__ __forceinline__ i64 gx_ldg_i8(const void* p, i64 i) { return (i64)__ldg((const signed char*)p + i); }
__device__ __forceinline__ i64 gx_ldg_u8(const void* p, i64 i) { return (i64)__ldg((const unsigned char*)p + i); }
__device__ __forceinline__ i64 gx_ldg_i16(const void* p, i64 i) { return (i64)__ldg((const short*)p + i); }
__device__ __forceinline__ i64 gx_ldg_u16(const void* p, i64 i) { return (i64)__ldg((const unsigned short*)p + i); }
__device__ __forceinline__ i64 gx_ldg_i32(const void* p, i64 i) { return (i64)__ldg((const int*)p + i); }
__device__ __forceinline__ i64 gx_ldg_u32(const void* p, i64 i) { return (i64)__ldg((const unsigned int*)p + i); }
__device__ __forceinline__ u64 gx_ldg_64(const void* p, i64 i) { return (u64)__ldg((const long long*)p + i); }
__device__ __forceinline__ u64 gx_ldg_f32(const void* p, i64 i) { return gx_B((double)__ldg((const float*)p + i)); }
__device__ __forceinline__ u64 gx_ldg_f32e(const void* p, i64 i) { return gxe_f2d(__ldg((const unsigned*)p + i)); }

// the same loads from a shared-memory staging buffer (staged filter kernel)
__device__ __forceinline__ i64 gx_lds_i8(const void* p, i64 i) { return (i64)((const signed char*)p)[i]; }
__device__ __forceinline__ i64 gx_lds_u8(const void* p, i64 i) { return (i64)((const unsigned char*)p)[i]; }
__device__ __forceinline__ i64 gx_lds_i16(const void* p, i64 i) { return (i64)((const short*)p)[i]; }
__device__ __forceinline__ i64 gx_lds_u16(const void* p, i64 i) { return (i64)((const unsigned short*)p)[i]; }
__device__ __forceinline__ i64 gx_lds_i32(const void* p, i64 i) { return (i64)((const int*)p)[i]; }
__device__ __forceinline__ i64 gx_lds_u32(const void* p, i64 i) { return (i64)((const unsigned int*)p)[i]; }
__device__ __forceinline__ u64 gx_lds_64(const void* p, i64 i) { return (u64)((const long long*)p)[i]; }
__device__ __forceinline__ u64 gx_lds_f32(const void* p, i64 i) { return gx_B((double)((const float*)p)[i]); }
__device__ __forceinline__ u64 gx_lds_f32e(const void* p, i64 i) { return gxe_f2d(((const unsigned*)p)[i]); }

// ---- bulk copies (TMA, 1-D) into shared memory with mbarrier completion ----
__device__ __forceinline__ u32 gx_saddr(const void* p) { return (u32)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void gx_mbar_init(u64* bar, u32 count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(gx_saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void gx_mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of bulk copies still to land
__device__ __forceinline__ void gx_mbar_arrive_tx(u64* bar, u32 bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(gx_saddr(bar)), "r"(bytes) : "memory");
}
// non-blocking test of the phase with the given parity
__device__ __forceinline__ bool gx_mbar_try_wait(u64* bar, u32 parity) {
  u32 ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(gx_saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
__device__ __forceinline__ void gx_bulk_g2s(void* dst, const void* src, u32 bytes, u64* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   gx_saddr(dst)),
               "l"(src), "r"(bytes), "r"(gx_saddr(bar))
               : "memory");
}
// 16-byte asynchronous global -> shared copy (L2 only), and an arrival on an
// mbarrier once every earlier copy of this thread has landed
__device__ __forceinline__ void gx_cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(gx_saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void gx_cp_arrive(u64* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(gx_saddr(bar)) : "memory");
}
// orders this thread's earlier generic-proxy accesses to shared memory before
// later bulk copies into it
__device__ __forceinline__ void gx_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// bounded wait for the phase of the given parity: each mbarrier.try_wait
// suspends the thread for at most about a microsecond (its time hint) unless
// the phase completes first; false once `max_polls` of them have failed (about
// max_polls microseconds) -- the caller then records an error instead of
// waiting forever
__device__ __forceinline__ bool gx_mbar_wait(u64* bar, u32 parity, u32 max_polls) {
  for (u32 i = 0; i < max_polls; i++) {
    u32 ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(gx_saddr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// one plain arrival on an mbarrier (release)
__device__ __forceinline__ void gx_mbar_arrive(u64* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(gx_saddr(bar)) : "memory");
}

// Named barrier 1 over `nthreads` threads (whole warps) that also ANDs a
// predicate over them: the consumer warps of the tile-staged kernels meet
// here without the producer and resolver warps.
__device__ __forceinline__ bool gx_bar_and(bool v, u32 nthreads) {
  u32 r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((u32)v), "r"(nthreads)
      : "memory");
  return r != 0u;
}

// ---- tile staging: the dynamic shared memory of the tile-staged kernels -----
// A tile's rows of every column a plan reads are copied here by bulk copies
// (one per column and tile); the kernels read them back by byte offset.
extern __shared__ __align__(128) unsigned char gx_smem[];
__device__ __forceinline__ i64 gx_sld_i8(u32 o) { return (i64)*(const signed char*)(gx_smem + o); }
__device__ __forceinline__ i64 gx_sld_u8(u32 o) { return (i64)*(const unsigned char*)(gx_smem + o); }
__device__ __forceinline__ i64 gx_sld_i16(u32 o) { return (i64)*(const short*)(gx_smem + o); }
__device__ __forceinline__ i64 gx_sld_u16(u32 o) { return (i64)*(const unsigned short*)(gx_smem + o); }
__device__ __forceinline__ i64 gx_sld_i32(u32 o) { return (i64)*(const int*)(gx_smem + o); }
__device__ __forceinline__ i64 gx_sld_u32(u32 o) { return (i64)*(const unsigned int*)(gx_smem + o); }
__device__ __forceinline__ u64 gx_sld_64(u32 o) { return (u64)*(const long long*)(gx_smem + o); }
__device__ __forceinline__ u64 gx_sld_f32(u32 o) { return gx_B((double)*(const float*)(gx_smem + o)); }
__device__ __forceinline__ u64 gx_sld_f32e(u32 o) { return gxe_f2d(*(const unsigned*)(gx_smem + o)); }

// Bulk copy of the bytes [lo, hi) of a column into shared memory at `dst`
// (16-byte aligned): the copy covers the 16-byte blocks that hold them, so it
// starts lo % 16 bytes early.  Every block copied holds at least one byte of
// [lo, hi), so no block reaches outside the pages that hold the column.
// Returns the bytes the copy moves (0 for an empty range); with issue false it
// only computes them.
__device__ __forceinline__ u32 gx_bulk_span(u32 dst, u64 lo, u64 hi, u64* bar, bool issue) {
  if (hi <= lo) return 0u;
  const u64 s = lo & ~15ull, e = (hi + 15ull) & ~15ull;
  const u32 bytes = (u32)(e - s);
  if (issue)
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(s), "r"(bytes), "r"(gx_saddr(bar))
                 : "memory");
  return bytes;
}

// Exclusive offset of warp `w`'s count among cnt[0..nw) (nw <= 32) and the
// total, computed by every lane of the calling warp from the shared counts.
__device__ __forceinline__ u32 gx_block_excl(const u32* cnt, int nw, u32* total, int w) {
  const int lane = threadIdx.x & 31;
  const u32 c = lane < nw ? cnt[lane] : 0u;
  u32 incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u32 t = __shfl_up_sync(GX_FULL, incl, d);
    if (lane >= d) incl += t;
  }
  *total = __shfl_sync(GX_FULL, incl, 31);
  return __shfl_sync(GX_FULL, incl - c, w & 31);
}

__device__ __forceinline__ void gx_st_8(void* p, i64 i, u64 v) { __stcs((signed char*)p + i, (signed char)v); }
__device__ __forceinline__ void gx_st_16(void* p, i64 i, u64 v) { __stcs((short*)p + i, (short)v); }
__device__ __forceinline__ void gx_st_32(void* p, i64 i, u64 v) { __stcs((int*)p + i, (int)v); }
__device__ __forceinline__ void gx_st_64(void* p, i64 i, u64 v) { __stcs((long long*)p + i, (long long)v); }
__device__ __forceinline__ void gx_st_f32(void* p, i64 i, u64 v) { __stcs((float*)p + i, (float)gx_D(v)); }

// ---- decoupled look-back (single-pass stable compaction) --------------------
// tile status word: bits 62..63 flag (0 none, 1 aggregate, 2 inclusive prefix),
// bits 0..61 value.
#define GX_ST_AGG (1ull << 62)
#define GX_ST_PFX (2ull << 62)
#define GX_ST_VAL ((1ull << 62) - 1ull)

__device__ __forceinline__ void gx_st_release(u64* p, u64 v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ u64 gx_ld_acquire(const u64* p) {
  u64 v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ u64 gx_ld_relaxed(const u64* p) {
  u64 v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Exclusive prefix of tile `tile` whose aggregate `agg` is already published
// (gx_tile_publish); called by one full warp; publishes the tile's inclusive
// prefix.
// Each poll reads a window of the 128 preceding status words (4 per lane,
// lane l holding distances 4l+1 .. 4l+4), sums the aggregates up to the
// nearest inclusive prefix, and moves 128 tiles further back while none is in
// the window -- with hundreds of tiles in flight the prefix frontier is that
// far back, so a wide window saves L2 round trips.  A status word carries its
// flag and value together, so relaxed loads suffice.  Waits are bounded: after
// `max_spins` polls without progress it records an error in *err and returns
// ~0ull (callers then skip their writes); a wait also ends early once *err is
// set by another tile.
__device__ __forceinline__ u64 gx_lookback_resolve(u64* status, i64 tile, u64 agg, int* err, u32 max_spins) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) return 0ull;  // published as a prefix already
  u64 excl = 0;
  i64 pred = tile - 1;  // distance 1
  u32 spins = 0;
  while (true) {
    u64 s[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const i64 idx = pred - (lane * 4 + i);
      s[i] = idx >= 0 ? gx_ld_relaxed(status + idx) : GX_ST_PFX;  // before tile 0: prefix 0
    }
    int first_pfx = 4;
#pragma unroll
    for (int i = 3; i >= 0; i--)
      if ((u32)(s[i] >> 62) == 2u) first_pfx = i;
    const u32 has_pfx = __ballot_sync(GX_FULL, first_pfx < 4);
    const int pl = has_pfx ? __ffs(has_pfx) - 1 : 0;
    const int pfx_i = __shfl_sync(GX_FULL, first_pfx, pl);
    // entries at window positions <= last (4 lane + i) are needed
    const int last = has_pfx ? pl * 4 + pfx_i : 127;
    bool missing = false;
    u64 v = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (lane * 4 + i <= last) {
        if ((u32)(s[i] >> 62) == 0u) missing = true;
        v += s[i] & GX_ST_VAL;
      }
    }
    if (__any_sync(GX_FULL, missing)) {
      if (++spins > max_spins) {
        if (lane == 0) atomicExch(err, 1);
        return ~0ull;
      }
      // another tile already gave up: its successors never complete, stop now
      if ((spins & 255u) == 0u && *(volatile int*)err != 0) return ~0ull;
      __nanosleep(32);
      continue;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GX_FULL, v, o);
    excl += v;
    if (has_pfx) break;
    pred -= 128;
  }
  if (lane == 0) gx_st_release(status + tile, GX_ST_PFX | (excl + agg));
  return excl;
}

// The same wait with a window of 32 x PER predecessors per poll (lane l reads
// distances PER l + 1 .. PER l + PER).  `known` / `known_incl`: a tile before
// `tile` whose inclusive prefix the caller already has (its block's previous
// tile; -1 and 0 when it has none): the walk treats it as a published prefix
// and never reads further back, so it spans at most the tiles other blocks
// claimed since.
template <int PER>
__device__ __forceinline__ u64 gx_lookback_wide(u64* status, i64 tile, u64 agg, int* err, u32 max_spins,
                                                i64 known = -1, u64 known_incl = 0ull) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) return 0ull;  // published as a prefix already
  u64 excl = 0;
  i64 pred = tile - 1;
  u32 spins = 0;
  while (true) {
    u64 s[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const i64 idx = pred - (lane * PER + i);
      s[i] = idx > known ? gx_ld_relaxed(status + idx) : (idx == known ? (GX_ST_PFX | known_incl) : GX_ST_PFX);
    }
    int first_pfx = PER;
#pragma unroll
    for (int i = PER - 1; i >= 0; i--)
      if ((u32)(s[i] >> 62) == 2u) first_pfx = i;
    const u32 has_pfx = __ballot_sync(GX_FULL, first_pfx < PER);
    const int pl = has_pfx ? __ffs(has_pfx) - 1 : 0;
    const int pfx_i = __shfl_sync(GX_FULL, first_pfx, pl);
    const int last = has_pfx ? pl * PER + pfx_i : 32 * PER - 1;
    bool missing = false;
    u64 v = 0;
#pragma unroll
    for (int i = 0; i < PER; i++) {
      if (lane * PER + i <= last) {
        if ((u32)(s[i] >> 62) == 0u) missing = true;
        v += s[i] & GX_ST_VAL;
      }
    }
    if (__any_sync(GX_FULL, missing)) {
      if (++spins > max_spins) {
        if (lane == 0) atomicExch(err, 1);
        return ~0ull;
      }
      if ((spins & 255u) == 0u && *(volatile int*)err != 0) return ~0ull;
      __nanosleep(200);  // a wide window re-read costs L2 bandwidth: poll less often
      continue;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GX_FULL, v, o);
    excl += v;
    if (has_pfx) break;
    pred -= 32 * PER;
  }
  if (lane == 0) gx_st_release(status + tile, GX_ST_PFX | (excl + agg));
  return excl;
}

// One non-blocking attempt at tile's exclusive prefix (aggregate `agg` already
// published), continuing from (*pred, *excl): walks back while the windows are
// complete; returns true with the prefix in *excl (and publishes the inclusive
// prefix), or false at the first tile that has not published yet, keeping the
// progress in *pred / *excl.  Called by one full warp; the values are
// warp-uniform.
__device__ __forceinline__ bool gx_lookback_poll(u64* status, i64 tile, u64 agg, i64* pred, u64* excl) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {  // published as a prefix already
    *excl = 0ull;
    return true;
  }
  i64 pr = *pred;
  u64 ex = *excl;
  while (true) {
    u64 s[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const i64 idx = pr - (lane * 4 + i);
      s[i] = idx >= 0 ? gx_ld_relaxed(status + idx) : GX_ST_PFX;
    }
    int first_pfx = 4;
#pragma unroll
    for (int i = 3; i >= 0; i--)
      if ((u32)(s[i] >> 62) == 2u) first_pfx = i;
    const u32 has_pfx = __ballot_sync(GX_FULL, first_pfx < 4);
    const int pl = has_pfx ? __ffs(has_pfx) - 1 : 0;
    const int pfx_i = __shfl_sync(GX_FULL, first_pfx, pl);
    const int last = has_pfx ? pl * 4 + pfx_i : 127;
    bool missing = false;
    u64 v = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (lane * 4 + i <= last) {
        if ((u32)(s[i] >> 62) == 0u) missing = true;
        v += s[i] & GX_ST_VAL;
      }
    }
    if (__any_sync(GX_FULL, missing)) {
      *pred = pr;
      *excl = ex;
      return false;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GX_FULL, v, o);
    ex += v;
    if (has_pfx) break;
    pr -= 128;
  }
  if (lane == 0) gx_st_release(status + tile, GX_ST_PFX | (ex + agg));
  *excl = ex;
  return true;
}

// Publishes a tile's aggregate (tile 0: its inclusive prefix) from the
// per-warp kept-row counts cnt[0..nw), writes each warp's exclusive offset
// within the tile to off[], and returns the tile's total; called by one full
// warp.
__device__ __forceinline__ u64 gx_tile_publish(u64* status, i64 tile, const u32* cnt, u64* off, int nw) {
  const int lane = threadIdx.x & 31;
  const u64 c = lane < nw ? (u64)cnt[lane] : 0ull;
  u64 incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u64 t = __shfl_up_sync(GX_FULL, incl, d);
    if (lane >= d) incl += t;
  }
  const u64 total = __shfl_sync(GX_FULL, incl, 31);
  if (lane < nw) off[lane] = incl - c;
  if (lane == 0) gx_st_release(status + tile, (tile == 0 ? GX_ST_PFX : GX_ST_AGG) | total);
  return total;
}

// Publish + resolve in one step (tile loops without a pipeline).
__device__ __forceinline__ u64 gx_lookback(u64* status, i64 tile, u64 agg, int* err, u32 max_spins) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) gx_st_release(status + tile, (tile == 0 ? GX_ST_PFX : GX_ST_AGG) | agg);
  return gx_lookback_resolve(status, tile, agg, err, max_spins);
}

// Appends `nbits` compressed validity bits to a warp's output bit stream.
// acc/fill are warp-uniform; full words inside the warp's own range are stored,
// words shared with a neighbouring range are OR-ed atomically (the mask was
// zeroed before the launch).
struct GxBitWriter {
  u64 acc;
  int fill;
  i64 word;     // output word index of acc's low 32 bits
  bool first;   // the first word may be shared with the previous range
  __device__ __forceinline__ void init(i64 start_bit) {
    acc = 0;
    fill = (int)(start_bit & 31);
    word = start_bit >> 5;
    first = fill != 0;
  }
  __device__ __forceinline__ void append(u32* mask, u32 bits, int nbits) {
    acc |= (u64)bits << fill;
    fill += nbits;
    if (fill >= 32) {
      if ((threadIdx.x & 31) == 0) {
        if (first) atomicOr(mask + word, (u32)acc);
        else mask[word] = (u32)acc;
      }
      first = false;
      acc >>= 32;
      fill -= 32;
      word++;
    }
  }
  __device__ __forceinline__ void flush(u32* mask) {
    if (fill > 0 && (threadIdx.x & 31) == 0) atomicOr(mask + word, (u32)acc);
  }
};

// ---------------------------------------------------------------- aggregation
// Global group table of the fused filter + aggregate kernel (structure of
// arrays over `cap` slots, cap a power of two).  A slot's state goes 0 (empty)
// -> 1 (claimed, keys being written) -> 2 (keys published).
struct GxAggArgs {
  u32* state;
  u32* nullm;                  // key null bits per slot
  u64* keys;                   // [key][cap]
  u64* acc;                    // [aggregation][cap]: sum bits / ordered min-max
  u64* cnt;                    // [aggregation][cap]: valid inputs
  u64* rows;                   // [cap]: rows per group
  u64 cap;
  int* overflow;               // set when a probe walked the whole table
  int* err;                    // set when a wait on a claimed slot gave up
  unsigned long long* groups;  // slots claimed
};

__device__ __forceinline__ u64 gx_mix64(u64 x) {
  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// binary64 bits -> a signed integer with the same order (min / max through
// integer atomics); the map is its own inverse
__device__ __forceinline__ long long gx_ord64(u64 b) {
  return (long long)(b ^ (((u64)((long long)b >> 63)) & 0x7FFFFFFFFFFFFFFFull));
}
__device__ __forceinline__ u64 gx_unord64(long long o) {
  return (u64)o ^ (((u64)(o >> 63)) & 0x7FFFFFFFFFFFFFFFull);
}

// Combining a value over the lanes of one peer set (lanes whose rows fall in
// the same group; every lane of the warp takes part, a lane outside any set
// being a set of its own).  Tree over the ranks within the set: at step s
// the survivors (ranks multiple of s) with a rank multiple of 2s take the
// partial of the survivor just above them.  After 5 steps rank 0 holds the
// combination of the whole set.  surv is the lane's peer mask.
struct GxPeers {
  u32 surv;
  int rank;
  __device__ __forceinline__ void init(u32 peers) {
    surv = peers;
    rank = __popc(peers & ((1u << (threadIdx.x & 31)) - 1u));
  }
  // the lane whose partial a receiver takes at step s (its own lane otherwise)
  __device__ __forceinline__ int partner() const {
    const int lane = threadIdx.x & 31;
    const u32 above = surv & ~((2u << lane) - 1u);
    return above ? __ffs(above) - 1 : lane;
  }
  __device__ __forceinline__ bool receives(int s) const {
    const int lane = threadIdx.x & 31;
    const u32 above = surv & ~((2u << lane) - 1u);
    return ((surv >> lane) & 1u) && ((rank / s) % 2 == 0) && above != 0u;
  }
  __device__ __forceinline__ void step(int s) {
    const int lane = threadIdx.x & 31;
    const bool stays = ((surv >> lane) & 1u) && ((rank / s) % 2 == 0);
    surv &= __ballot_sync(0xffffffffu, stays);
  }
};
