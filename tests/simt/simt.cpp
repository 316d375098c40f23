// Execution of CUDA kernels on the host for the engine's CPU checks.
//
// A block's threads are fibers that run until they reach
// __syncthreads or a warp collective; a collective resolves once all 32
// lanes of the warp wait at the same one (anything else is reported as a
// divergence error), a barrier once every live thread of the block waits.
// Warps of a block run in ascending order, or descending with
// SIMT_REVERSE=1, so data that one warp reads before another has written it
// without a barrier shows up.  Blocks are spread over host threads
// (SIMT_THREADS, default: all cores).  Every device allocation ends right
// below a PROT_NONE page and starts filled with 0xa5 bytes (device memory
// is not zeroed); freed allocations become PROT_NONE: an out-of-range or
// stale access faults at once, and the fault report names the kernel, the
// block and the nearest allocation.
#include <signal.h>
#include <sys/mman.h>
#include <setjmp.h>
#include <ucontext.h>
#include <unistd.h>

#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "cuda_runtime.h"

namespace simt {

enum State { READY, WAIT_WARP, WAIT_BAR, DONE };
// A fiber starts on its own stack through makecontext/swapcontext; every
// later switch uses _setjmp/_longjmp, which save no signal mask (no system
// call per switch).
struct Fiber {
  uint3 tid;
  ucontext_t ctx;
  jmp_buf jb;
  bool made = false, started = false;
  int state, op;
  unsigned mask;
  unsigned long long v;
  int arg;
  unsigned long long res;
  char* stack = nullptr;
};

thread_local uint3 g_tid, g_bid;
dim3 g_bdim, g_gdim;
static thread_local Fiber* g_cur = nullptr;
static thread_local ucontext_t g_sched_uc;
static thread_local jmp_buf g_sched;
static thread_local std::vector<Fiber>* g_fibers = nullptr;
static CallFn g_fn = nullptr;
static void* g_obj = nullptr;
static const char* g_name = "";
static const size_t kStack = 128 * 1024;
static long long g_launches = 0;
static const bool g_reverse = getenv("SIMT_REVERSE") != nullptr;
static int g_nthreads = getenv("SIMT_THREADS") ? atoi(getenv("SIMT_THREADS")) : (int)sysconf(_SC_NPROCESSORS_ONLN);

static void die(const char* what) {
  std::fprintf(stderr, "SIMT ERROR: %s in kernel %s block %u thread %u\n", what, g_name, g_bid.x, g_cur ? g_cur->tid.x : 0u);
  std::fflush(stderr);
  _exit(98);
}

static void trampoline() {
  g_fn(g_obj);
  g_cur->state = DONE;
  _longjmp(g_sched, 1);
}

static inline void yield() {
  if (!_setjmp(g_cur->jb)) _longjmp(g_sched, 1);
}

static inline void resume(Fiber& f) {
  if (_setjmp(g_sched)) return;
  if (!f.started) {
    f.started = true;
    swapcontext(&g_sched_uc, &f.ctx);
  } else {
    _longjmp(f.jb, 1);
  }
}

void syncthreads() {
  g_cur->state = WAIT_BAR;
  yield();
}

unsigned long long collective(int op, unsigned mask, unsigned long long v, int arg) {
  Fiber* f = g_cur;
  f->state = WAIT_WARP;
  f->op = op;
  f->mask = mask;
  f->v = v;
  f->arg = arg;
  yield();
  return f->res;
}

static void init_fiber(Fiber& f, unsigned t) {
  f.tid = uint3{t, 0, 0};
  f.state = READY;
  f.started = false;
  if (!f.stack) {
    f.stack = (char*)mmap(nullptr, kStack + 4096, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (f.stack == MAP_FAILED) die("stack mmap");
    mprotect(f.stack, 4096, PROT_NONE);  // stack overflow guard
  }
  if (!f.made) {
    getcontext(&f.ctx);
    f.made = true;
  }
  f.ctx.uc_stack.ss_sp = f.stack + 4096;
  f.ctx.uc_stack.ss_size = kStack;
  f.ctx.uc_link = nullptr;
  makecontext(&f.ctx, trampoline, 0);
}

static void resolve_warp(Fiber* w, int nl) {
  int op = -1;
  unsigned mask = 0;
  for (int l = 0; l < nl; ++l) {
    if (op < 0) {
      op = w[l].op;
      mask = w[l].mask;
    } else if (w[l].op != op || w[l].mask != mask) {
      g_cur = &w[l];
      die("warp collective: lanes at different collectives");
    }
  }
  if (mask != 0xffffffffu || nl != 32) {
    g_cur = &w[0];
    die("warp collective without all 32 lanes");
  }
  unsigned long long res[32];
  switch (op) {
    case OP_SHFL:
      for (int l = 0; l < 32; ++l) res[l] = w[w[l].arg & 31].v;
      break;
    case OP_SHFL_UP:
      for (int l = 0; l < 32; ++l) res[l] = (l - w[l].arg >= 0) ? w[l - w[l].arg].v : w[l].v;
      break;
    case OP_SHFL_XOR:
      for (int l = 0; l < 32; ++l) res[l] = w[(l ^ w[l].arg) & 31].v;
      break;
    case OP_BALLOT:
    case OP_ANY: {
      unsigned b = 0;
      for (int l = 0; l < 32; ++l)
        if (w[l].v) b |= 1u << l;
      for (int l = 0; l < 32; ++l) res[l] = op == OP_BALLOT ? b : (b != 0);
      break;
    }
    case OP_MATCH_ANY:
      for (int l = 0; l < 32; ++l) {
        unsigned b = 0;
        for (int k = 0; k < 32; ++k)
          if (w[k].v == w[l].v) b |= 1u << k;
        res[l] = b;
      }
      break;
    default:
      die("unknown collective");
  }
  for (int l = 0; l < 32; ++l) {
    w[l].res = res[l];
    w[l].state = READY;
  }
}

static void run_block(unsigned b, int T) {
  if (!g_fibers) {
    // a ucontext_t points into itself: the fibers must never move
    g_fibers = new std::vector<Fiber>();
    g_fibers->reserve(1024);
  }
  std::vector<Fiber>& fib = *g_fibers;
  if ((int)fib.size() < T) fib.resize(T);
  const int nw = (T + 31) / 32;
  g_bid = uint3{b % g_gdim.x, b / g_gdim.x, 0};  // blocks run by linear index, x fastest
  for (int t = 0; t < T; ++t) init_fiber(fib[t], (unsigned)t);
  int done = 0;
  for (;;) {
    bool progress = false;
    for (int wj = 0; wj < nw; ++wj) {
      const int wi = g_reverse ? nw - 1 - wj : wj;
      Fiber* w = &fib[wi * 32];
      const int nl = std::min(32, T - wi * 32);
      for (;;) {
        bool ran = false;
        for (int l = 0; l < nl; ++l) {
          if (w[l].state != READY) continue;
          g_cur = &w[l];
          g_tid = w[l].tid;
          resume(w[l]);
          g_cur = nullptr;
          ran = true;
          if (w[l].state == DONE) ++done;
        }
        if (ran) progress = true;
        int nwait = 0, ndone = 0, nbar = 0;
        for (int l = 0; l < nl; ++l) {
          nwait += w[l].state == WAIT_WARP;
          ndone += w[l].state == DONE;
          nbar += w[l].state == WAIT_BAR;
        }
        if (nwait > 0 && nwait == nl) {
          resolve_warp(w, nl);
          progress = true;
          continue;
        }
        if (nwait > 0 && nwait + ndone == nl) {
          g_cur = &w[0];
          die("warp collective with an exited lane");
        }
        if (nwait > 0 && nbar > 0) {
          g_cur = &w[0];
          die("lanes of one warp at a barrier and at a collective");
        }
        break;
      }
    }
    if (done == T) break;
    int nbar = 0, nready = 0;
    for (int t = 0; t < T; ++t) {
      nbar += fib[t].state == WAIT_BAR;
      nready += fib[t].state == READY;
    }
    if (nbar > 0 && nbar + done == T) {
      for (int t = 0; t < T; ++t)
        if (fib[t].state == WAIT_BAR) fib[t].state = READY;
      continue;
    }
    if (!progress && nready == 0) {
      g_cur = &fib[0];
      die("deadlock: threads wait at different barriers or collectives");
    }
  }
}

// persistent worker threads (their fibers and stacks are reused)
static std::mutex g_pm;
static std::condition_variable g_pcv, g_pdone;
static long long g_gen = 0;
static unsigned g_pgrid = 0;
static int g_pT = 0, g_pactive = 0;
static std::atomic<unsigned> g_next{0};
static std::vector<std::thread>* g_workers = nullptr;

static void worker() {
  long long seen = 0;
  for (;;) {
    unsigned grid;
    int T;
    {
      std::unique_lock<std::mutex> lk(g_pm);
      g_pcv.wait(lk, [&] { return g_gen != seen; });
      seen = g_gen;
      grid = g_pgrid;
      T = g_pT;
    }
    for (;;) {
      const unsigned b = g_next.fetch_add(1);
      if (b >= grid) break;
      run_block(b, T);
    }
    std::lock_guard<std::mutex> lk(g_pm);
    if (--g_pactive == 0) g_pdone.notify_all();
  }
}

void launch_impl(const char* name, dim3 grid, dim3 block, CallFn fn, void* obj) {
  g_name = name;
  if (grid.z != 1 || block.y != 1 || block.z != 1) die("only 1-D blocks and 1-D or 2-D grids are supported");
  if (block.x == 0 || block.x > 1024) die("bad block size");
  ++g_launches;
  g_fn = fn;
  g_obj = obj;
  g_gdim = grid;
  g_bdim = block;
  const int T = (int)block.x;
  const unsigned nblocks = grid.x * grid.y;
  if (g_nthreads <= 1 || nblocks == 1) {
    for (unsigned b = 0; b < nblocks; ++b) run_block(b, T);
  } else {
    std::unique_lock<std::mutex> lk(g_pm);
    if (!g_workers) {
      g_workers = new std::vector<std::thread>();
      for (int i = 0; i < g_nthreads; ++i) g_workers->emplace_back(worker);
      for (auto& t : *g_workers) t.detach();
    }
    g_pgrid = nblocks;
    g_pT = T;
    g_next = 0;
    g_pactive = (int)g_workers->size();
    ++g_gen;
    g_pcv.notify_all();
    g_pdone.wait(lk, [] { return g_pactive == 0; });
  }
  g_name = "";
}

long long launches() { return g_launches; }

// ------------------------------------------------------------------ memory
struct Alloc {
  char* base;
  size_t maplen;
  char* user;
  size_t bytes;
  bool live;
};
static std::map<uintptr_t, Alloc> g_allocs;
static std::mutex g_am;

void* dev_alloc(size_t bytes) {
  const size_t ps = 4096;
  size_t rb = (bytes + 15) / 16 * 16;
  if (rb == 0) rb = 16;
  const size_t body = (rb + ps - 1) / ps * ps, maplen = body + 2 * ps;
  char* base = (char*)mmap(nullptr, maplen, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (base == MAP_FAILED) return nullptr;
  mprotect(base, ps, PROT_NONE);
  mprotect(base + ps + body, ps, PROT_NONE);
  char* user = base + ps + body - rb;
  std::memset(user, 0xa5, rb);
  std::lock_guard<std::mutex> g(g_am);
  g_allocs[(uintptr_t)user] = Alloc{base, maplen, user, bytes, true};
  return user;
}

void dev_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> g(g_am);
  auto it = g_allocs.find((uintptr_t)p);
  if (it == g_allocs.end() || !it->second.live) {
    std::fprintf(stderr, "SIMT ERROR: free of an unknown device pointer %p\n", p);
    _exit(97);
  }
  it->second.live = false;
  mprotect(it->second.base, it->second.maplen, PROT_NONE);
  madvise(it->second.base, it->second.maplen, MADV_DONTNEED);
}

static void on_fault(int sig, siginfo_t* si, void*) {
  std::fprintf(stderr, "SIMT FAULT: signal %d at %p in kernel '%s' block %u thread %u (launch %lld)\n", sig, si->si_addr,
               g_name, g_bid.x, g_cur ? g_cur->tid.x : 0u, g_launches);
  const uintptr_t a = (uintptr_t)si->si_addr;
  const Alloc* best = nullptr;
  long long bd = 0;
  for (auto& kv : g_allocs) {
    const Alloc& x = kv.second;
    const uintptr_t lo = (uintptr_t)x.base, hi = lo + x.maplen;
    const long long dd = a < lo ? (long long)(lo - a) : a >= hi ? (long long)(a - hi) : 0;
    if (!best || dd < bd) {
      best = &x;
      bd = dd;
    }
  }
  if (best)
    std::fprintf(stderr, "  nearest allocation: %zu bytes at %p (%s), offset %lld\n", best->bytes, (void*)best->user,
                 best->live ? "live" : "freed", (long long)(a - (uintptr_t)best->user));
  std::fflush(stderr);
  _exit(99);
}

struct Init {
  Init() {
    static char altstack[1 << 16];
    stack_t ss;
    ss.ss_sp = altstack;
    ss.ss_size = sizeof(altstack);
    ss.ss_flags = 0;
    sigaltstack(&ss, nullptr);
    struct sigaction sa;
    std::memset(&sa, 0, sizeof(sa));
    sa.sa_sigaction = on_fault;
    sa.sa_flags = SA_SIGINFO | SA_ONSTACK;
    sigaction(SIGSEGV, &sa, nullptr);
    sigaction(SIGBUS, &sa, nullptr);
  }
} g_init;

}  // namespace simt

cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
// the host stand-in reports a GB300's 152 SMs, so persistent grids have the
// device's block count
cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr, int) {
  *v = 152;
  return cudaSuccess;
}
const char* cudaGetErrorString(cudaError_t e) { return e ? "simt error" : "no error"; }
cudaError_t cudaGetLastError() { return cudaSuccess; }
cudaError_t cudaMemPoolCreate(cudaMemPool_t* p, const cudaMemPoolProps*) {
  *p = (cudaMemPool_t)0x1;
  return cudaSuccess;
}
cudaError_t cudaMemPoolDestroy(cudaMemPool_t) { return cudaSuccess; }
cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t, cudaMemPoolAttr, void*) { return cudaSuccess; }
cudaError_t cudaMallocFromPoolAsync(void** p, size_t bytes, cudaMemPool_t, cudaStream_t) {
  *p = simt::dev_alloc(bytes);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFreeAsync(void* p, cudaStream_t) {
  simt::dev_free(p);
  return cudaSuccess;
}
cudaError_t cudaMalloc(void** p, size_t bytes) {
  *p = simt::dev_alloc(bytes);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
  simt::dev_free(p);
  return cudaSuccess;
}
cudaError_t cudaMallocHost(void** p, size_t bytes) {
  *p = std::malloc(bytes ? bytes : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFreeHost(void* p) {
  std::free(p);
  return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t) {
  std::memset(d, v, n);
  return cudaSuccess;
}
cudaError_t cudaMemset(void* d, int v, size_t n) {
  std::memset(d, v, n);
  return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
// one device, and every launch runs to completion on the calling thread: a
// stream is only a distinct handle
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned) {
  *s = (cudaStream_t) new char[1];
  return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
  delete[] (char*)s;
  return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* e) {
  *e = (cudaEvent_t)0x1;
  return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.f;
  return cudaSuccess;
}
