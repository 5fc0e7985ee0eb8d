// Host side of the graph-specialised f32 layered decoder (layered_nr.cuh).
//
// Two builds of one kernel source:
//   * compiled here by nvcc, once per base graph, with Z and the shifts read from the
//     launch parameters: serves every code of the base graph;
//   * compiled at run time for one code, with Z and every shift as constants, so that
//     each edge address is an immediate offset and each lifted row's state address a
//     constant: fewer instructions per edge update, the same results.  The compiler is the
//     CUDA toolkit's nvcc when one is found (its front end gives this kernel about 5 %
//     faster code than NVRTC's, measured on GB300), else NVRTC.  The cubin is kept for the
//     process (per base graph and lifting size) and on disk (keyed by a hash of the
//     sources, the options and the compiler), and loaded with the runtime's library API.
//     Without a compiler, or if it fails, the nvcc build above runs.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <fcntl.h>
#include <nvrtc.h>
#include <spawn.h>
#include <sys/stat.h>
#include <sys/wait.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

extern char** environ;  // passed to the compiler process

#include "nr_decode.h"
#include "nr_jit_sources.inc"  // generated by build.py: the kernel source files as text

namespace cbk {
namespace {

const void* generic_kernel(int bg, bool learned) {
  if (learned)
    return bg == 1 ? (const void*)&cbn::layered_nr_kernel<1, cbn::RuntimeLifting, cbn::NrLearnedArgs>
                   : (const void*)&cbn::layered_nr_kernel<2, cbn::RuntimeLifting, cbn::NrLearnedArgs>;
  return bg == 1 ? (const void*)&cbn::layered_nr_kernel<1, cbn::RuntimeLifting>
                 : (const void*)&cbn::layered_nr_kernel<2, cbn::RuntimeLifting>;
}

// the entries of `h` in the order of the compile-time base graph (row-major, as the
// standard's tables list them)
bool matches_base_graph(const cbh::NrCode& h) {
  const int* start = h.bg == 1 ? cbn::BaseGraph1::start : cbn::BaseGraph2::start;
  const int* col = h.bg == 1 ? cbn::BaseGraph1::col : cbn::BaseGraph2::col;
  const int rows = h.bg == 1 ? cbn::BaseGraph1::rows : cbn::BaseGraph2::rows;
  if (h.rows_n != rows || (int)h.layer_start.size() != rows + 1) return false;
  for (int i = 0; i <= rows; i++)
    if (h.layer_start[i] != start[i]) return false;
  for (int t = 0; t < start[rows]; t++)
    if (h.entry_col[t] != col[t]) return false;
  return true;
}

// ---- the run-time compiler, loaded on first use
struct Nvrtc {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcVersion) version = nullptr;
  std::string why;  // empty when usable
};

const Nvrtc& nvrtc() {
  static Nvrtc api = [] {
    Nvrtc a;
    if (const char* off = std::getenv("COMRS_NO_JIT")) {
      if (*off && std::strcmp(off, "0") != 0) {
        a.why = "COMRS_NO_JIT is set";
        return a;
      }
    }
    void* h = nullptr;
    for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"})
      if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
      a.why = "libnvrtc.so.13 not found";
      return a;
    }
    a.create = (decltype(a.create))dlsym(h, "nvrtcCreateProgram");
    a.compile = (decltype(a.compile))dlsym(h, "nvrtcCompileProgram");
    a.log_size = (decltype(a.log_size))dlsym(h, "nvrtcGetProgramLogSize");
    a.log = (decltype(a.log))dlsym(h, "nvrtcGetProgramLog");
    a.cubin_size = (decltype(a.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
    a.cubin = (decltype(a.cubin))dlsym(h, "nvrtcGetCUBIN");
    a.destroy = (decltype(a.destroy))dlsym(h, "nvrtcDestroyProgram");
    a.version = (decltype(a.version))dlsym(h, "nvrtcVersion");
    if (!a.create || !a.compile || !a.log_size || !a.log || !a.cubin_size || !a.cubin || !a.destroy || !a.version)
      a.why = "libnvrtc lacks an entry point";
    return a;
  }();
  return api;
}

const char* const kJitOptions[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=false"};
// nvcc's, for the same code
const char* const kNvccOptions[] = {"-cubin", "-O3", "-std=c++17", "-arch=sm_103a", "-fmad=false",
                                    "--expt-relaxed-constexpr"};

// The toolkit's nvcc: $COMRS_NVCC if set (empty: none), else $CUDA_HOME/bin/nvcc,
// /usr/local/cuda/bin/nvcc or the first on PATH; empty when none is found or COMRS_NO_JIT
// is set.
const std::string& nvcc_path() {
  static const std::string path = [] {
    if (const char* off = std::getenv("COMRS_NO_JIT"))
      if (*off && std::strcmp(off, "0") != 0) return std::string();
    std::vector<std::string> cand;
    // a set COMRS_NVCC names the compiler, or (empty) turns nvcc off: NVRTC compiles
    if (const char* p = std::getenv("COMRS_NVCC"))
      return std::string(*p && access(p, X_OK) == 0 ? p : "");
    if (const char* p = std::getenv("CUDA_HOME")) cand.push_back(std::string(p) + "/bin/nvcc");
    cand.push_back("/usr/local/cuda/bin/nvcc");
    if (const char* p = std::getenv("PATH")) {
      std::string s = p;
      for (size_t a = 0; a <= s.size();) {
        size_t b = s.find(':', a);
        if (b == std::string::npos) b = s.size();
        if (b > a) cand.push_back(s.substr(a, b - a) + "/nvcc");
        a = b + 1;
      }
    }
    for (const std::string& c : cand)
      if (!c.empty() && access(c.c_str(), X_OK) == 0) return c;
    return std::string();
  }();
  return path;
}

// the code's own kernel: Z, the shifts (row-major) and the min-sum rule as constants; the
// plain decoder or the learned min-sum (which has no rule of its own)
std::string jit_source(const cbh::NrCode& h, bool learned, int rule) {
  std::ostringstream s;
  s << "#include \"layered_nr.cuh\"\nnamespace cbn {\nstruct FixedLifting {\n"
    << "  static constexpr bool fixed = true;\n  static constexpr int z = " << h.z << ";\n"
    << "  static constexpr int shift[" << h.entry_shift.size() << "] = {";
  for (size_t t = 0; t < h.entry_shift.size(); t++) s << (t ? ", " : "") << h.entry_shift[t];
  s << "};\n  static constexpr int rule = " << (learned ? 1 : rule) << ";\n};\n}  // namespace cbn\n";
  const char* P = learned ? "cbn::NrLearnedArgs" : "cbn::NrArgs";
  s << "template __global__ void cbn::layered_nr_kernel<" << h.bg << ", cbn::FixedLifting, " << P
    << ">(const __grid_constant__ " << P << ");\n";
  return s.str();
}

uint64_t fnv1a(uint64_t h, const std::string& s) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 0x100000001b3ull;
  }
  return h;
}

std::string cache_key(const cbh::NrCode& h, const std::string& src) {
  uint64_t k = fnv1a(0xcbf29ce484222325ull, src);
  for (int i = 0; i < kJitFileCount; i++) k = fnv1a(fnv1a(k, kJitFileNames[i]), kJitFileTexts[i]);
  for (const char* o : kJitOptions) k = fnv1a(k, o);
  for (const char* o : kNvccOptions) k = fnv1a(k, o);
  // the compiler: nvcc (its path and file's size and time) or NVRTC (its version)
  const std::string& nv = nvcc_path();
  struct stat sb;
  if (!nv.empty() && stat(nv.c_str(), &sb) == 0) {
    k = fnv1a(k, nv + ":" + std::to_string((long long)sb.st_size) + ":" + std::to_string((long long)sb.st_mtime));
  } else {
    int ma = 0, mi = 0;
    if (nvrtc().version) nvrtc().version(&ma, &mi);
    k = fnv1a(k, "nvrtc " + std::to_string(ma) + "." + std::to_string(mi));
  }
  char buf[96];
  std::snprintf(buf, sizeof buf, "nr_bg%d_z%d_%016llx.cubin", h.bg, h.z, (unsigned long long)k);
  return buf;
}

// <directory of this library>/_build/jit (or $COMRS_JIT_CACHE); empty if unknown
std::string cache_dir() {
  if (const char* d = std::getenv("COMRS_JIT_CACHE")) return d;
  Dl_info info;
  if (!dladdr((const void*)&cache_dir, &info) || !info.dli_fname) return "";
  std::string p = info.dli_fname;
  const size_t slash = p.rfind('/');
  return (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/_build/jit";
}

bool read_file(const std::string& path, std::vector<char>& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  const bool ok = n > 0 && std::fread(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok;
}

void write_file(const std::string& dir, const std::string& name, const std::vector<char>& data) {
  if (dir.empty()) return;
  // mkdir -p of the last two components (_build/jit); failures leave the cache unused
  const size_t slash = dir.rfind('/');
  if (slash != std::string::npos) mkdir(dir.substr(0, slash).c_str(), 0755);
  mkdir(dir.c_str(), 0755);
  const std::string tmp = dir + "/." + name + "." + std::to_string(getpid());
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return;
  const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
  std::fclose(f);
  if (ok) std::rename(tmp.c_str(), (dir + "/" + name).c_str());
  else std::remove(tmp.c_str());
}

// nvcc on the sources written to a private temporary directory (no shell: posix_spawn)
bool compile_nvcc(const std::string& nvcc, const std::string& src, std::vector<char>& cubin, std::string* note) {
  const char* tmp = std::getenv("TMPDIR");
  std::string tmpl = std::string(tmp && *tmp ? tmp : "/tmp") + "/comrs_jit_XXXXXX";
  std::vector<char> buf(tmpl.begin(), tmpl.end());
  buf.push_back('\0');
  if (!mkdtemp(buf.data())) {
    if (note) *note = "no temporary directory for nvcc";
    return false;
  }
  const std::string dir = buf.data();
  std::vector<std::string> files;
  auto put = [&](const std::string& name, const char* text) {
    const std::string path = dir + "/" + name;
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t n = std::strlen(text);
    const bool ok = std::fwrite(text, 1, n, f) == n;
    std::fclose(f);
    files.push_back(path);
    return ok;
  };
  bool ok = put("nr_code.cu", src.c_str());
  for (int i = 0; ok && i < kJitFileCount; i++) ok = put(kJitFileNames[i], kJitFileTexts[i]);
  const std::string out = dir + "/nr_code.cubin", log = dir + "/nvcc.log", inc = "-I" + dir,
                    in = dir + "/nr_code.cu";
  if (ok) {
    std::vector<const char*> argv = {nvcc.c_str()};
    for (const char* o : kNvccOptions) argv.push_back(o);
    for (const char* a : {inc.c_str(), in.c_str(), "-o", out.c_str()}) argv.push_back(a);
    argv.push_back(nullptr);
    posix_spawn_file_actions_t fa;
    posix_spawn_file_actions_init(&fa);
    posix_spawn_file_actions_addopen(&fa, 1, log.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    posix_spawn_file_actions_adddup2(&fa, 1, 2);
    pid_t pid = 0;
    int status = 0;
    ok = posix_spawn(&pid, nvcc.c_str(), &fa, nullptr, const_cast<char* const*>(argv.data()), environ) == 0 &&
         waitpid(pid, &status, 0) == pid && WIFEXITED(status) && WEXITSTATUS(status) == 0;
    posix_spawn_file_actions_destroy(&fa);
    ok = ok && read_file(out, cubin);
    if (!ok && note) {
      std::vector<char> text;
      read_file(log, text);
      *note = "nvcc failed: " + std::string(text.begin(), text.end()).substr(0, 400);
    }
  }
  files.push_back(out);
  files.push_back(log);
  for (const std::string& f : files) std::remove(f.c_str());
  rmdir(dir.c_str());
  return ok;
}

bool compile_nvrtc(const cbh::NrCode& h, const std::string& src, std::vector<char>& cubin, std::string* note) {
  const Nvrtc& api = nvrtc();
  if (!api.why.empty()) {
    if (note) *note = api.why;
    return false;
  }
  nvrtcProgram prog = nullptr;
  if (api.create(&prog, src.c_str(), "nr_code.cu", kJitFileCount, kJitFileTexts, kJitFileNames) != NVRTC_SUCCESS) {
    if (note) *note = "nvrtcCreateProgram failed";
    return false;
  }
  const nvrtcResult r = api.compile(prog, (int)(sizeof kJitOptions / sizeof *kJitOptions), kJitOptions);
  bool ok = r == NVRTC_SUCCESS;
  size_t n = 0;
  if (ok && api.cubin_size(prog, &n) == NVRTC_SUCCESS && n > 0) {
    cubin.resize(n);
    ok = api.cubin(prog, cubin.data()) == NVRTC_SUCCESS;
  } else {
    ok = false;
  }
  if (!ok && note) {
    size_t ls = 0;
    api.log_size(prog, &ls);
    std::string log(ls, '\0');
    if (ls) api.log(prog, &log[0]);
    *note = "NVRTC failed for BG" + std::to_string(h.bg) + " Z=" + std::to_string(h.z) + ": " + log.substr(0, 400);
  }
  api.destroy(&prog);
  return ok;
}

// the code's specialisation: nvcc if found, else NVRTC
bool compile(const cbh::NrCode& h, const std::string& src, std::vector<char>& cubin, std::string* note) {
  const std::string& nv = nvcc_path();
  std::string why;
  if (!nv.empty() && compile_nvcc(nv, src, cubin, &why)) return true;
  if (compile_nvrtc(h, src, cubin, note)) return true;
  if (note && !why.empty()) *note = why + "; " + *note;
  return false;
}

// the specialised kernels of this process, by cache key
std::mutex g_jit_mu;
std::map<std::string, cudaKernel_t> g_jit_kernels;
std::map<std::pair<cudaKernel_t, int>, size_t> g_jit_smem_set;  // (kernel, device) -> dynamic smem set

}  // namespace

// the learned kernel's launch parameters stay within the 32,764 bytes a launch takes
static_assert(sizeof(cbn::NrLearnedArgs) <= 32764, "NrLearnedArgs exceeds the launch parameter limit");

void fill_nr_args(const cbh::NrCode& h, cbn::NrArgs& a) {
  std::memset(&a, 0, sizeof a);
  a.z = h.z;
  a.n_full = h.n_full;
  a.k = h.k;
  a.k_info = h.k_info;
  a.e = h.e;
  a.rows = h.rows_n;
  a.n_entries = (int)h.entry_col.size();
  a.map_kind = h.map_is_offset ? 0 : (h.has_repeats ? 2 : 1);
  for (int t = 0; t < a.n_entries; t++) {
    a.entry[t] = ((uint32_t)h.entry_col[t] << 16) | h.entry_shift[t];
    a.eaddr[t].x = 4u * h.entry_shift[t];
    a.eaddr[t].y = 4u * (uint32_t)h.entry_col[t] * (uint32_t)h.z;
  }
  for (int i = 0; i <= h.rows_n; i++) a.layer_start[i] = (uint16_t)h.layer_start[i];
}

size_t nr_smem(const cbh::NrCode& h) {
  return cbn::nr_smem_bytes(h.n_full, h.z, h.rows_n, (int)h.entry_col.size());
}

bool nr_prepare(const cbh::NrCode& h, std::string* note, bool learned, int rule) {
  if (!matches_base_graph(h)) {
    if (note) *note = "entries not in the base graph's order";
    return false;
  }
  const std::string src = jit_source(h, learned, rule);
  const std::string key = cache_key(h, src), dir = cache_dir();
  std::vector<char> cubin;
  if (!dir.empty() && read_file(dir + "/" + key, cubin)) return true;
  if (!compile(h, src, cubin, note)) return false;
  write_file(dir, key, cubin);
  return true;
}

NrKernel nr_kernel(const cbh::NrCode& h, int device, bool specialize, std::string* note, bool learned, int rule) {
  NrKernel k;
  k.fn = generic_kernel(h.bg, learned);
  if (!matches_base_graph(h)) {
    k.fn = nullptr;
    if (note) *note = "entries not in the base graph's order";
    return k;
  }
  if (!specialize) return k;
  const std::string src = jit_source(h, learned, rule);
  const std::string key = cache_key(h, src);
  std::lock_guard<std::mutex> lock(g_jit_mu);
  auto it = g_jit_kernels.find(key);
  if (it == g_jit_kernels.end()) {
    const std::string dir = cache_dir();
    std::vector<char> cubin;
    const bool cached = !dir.empty() && read_file(dir + "/" + key, cubin);
    if (!cached && !compile(h, src, cubin, note)) return k;
    cudaLibrary_t lib = nullptr;
    if (cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
      cudaGetLastError();
      if (note) *note = "cudaLibraryLoadData failed for the specialised decoder";
      return k;
    }
    unsigned int count = 0;
    cudaKernel_t kern = nullptr;
    if (cudaLibraryGetKernelCount(&count, lib) != cudaSuccess || count != 1 ||
        cudaLibraryEnumerateKernels(&kern, 1, lib) != cudaSuccess) {
      cudaGetLastError();
      if (note) *note = "the specialised library does not hold one kernel";
      return k;
    }
    if (!cached) write_file(dir, key, cubin);
    it = g_jit_kernels.emplace(key, kern).first;
  }
  k.fn = (const void*)it->second;
  k.specialized = true;
  k.library = true;
  (void)device;
  return k;
}

namespace {
cudaError_t set_smem(const NrKernel& k, size_t smem, int device) {
  if (!k.library) return cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  std::lock_guard<std::mutex> lock(g_jit_mu);
  const auto key = std::make_pair((cudaKernel_t)k.fn, device);
  auto it = g_jit_smem_set.find(key);
  if (it != g_jit_smem_set.end() && it->second == smem) return cudaSuccess;
  const cudaError_t e = cudaKernelSetAttributeForDevice((cudaKernel_t)k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)smem, device);
  if (e == cudaSuccess) g_jit_smem_set[key] = smem;
  return e;
}
}  // namespace

namespace {
// resident CTAs of a kernel of this code's block size with `smem` bytes of shared memory
int grid_for(const NrKernel& k, const cbh::NrCode& h, int device, size_t smem) {
  if (set_smem(k, smem, device) != cudaSuccess) return 0;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, ((h.z + 31) / 32) * 32, smem) != cudaSuccess)
    return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return per_sm * sms;
}
}  // namespace

int nr_grid_size(const NrKernel& k, const cbh::NrCode& h, int device) { return grid_for(k, h, device, nr_smem(h)); }

int nr_learned_grid_size(const NrKernel& k, const cbh::NrCode& h, int device) {
  return grid_for(k, h, device, cbn::nr_learned_smem_bytes(h.n_full, h.z, h.rows_n, (int)h.entry_col.size()));
}

namespace {
// one launch of the decoder for lifting z with `smem` bytes of shared memory; `params`
// points at its launch parameters (NrArgs or NrLearnedArgs)
cudaError_t launch_with(const NrKernel& k, const void* params, int z, size_t smem, int grid, cudaStream_t stream) {
  int device = 0;
  cudaGetDevice(&device);
  cudaError_t e = set_smem(k, smem, device);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<void*>(params)};
  return cudaLaunchKernel(k.fn, dim3(grid), dim3(((z + 31) / 32) * 32), args, smem, stream);
}
}  // namespace

cudaError_t nr_launch(const NrKernel& k, const cbn::NrArgs& a, int grid, cudaStream_t stream) {
  return launch_with(k, &a, a.z, cbn::nr_smem_bytes(a.n_full, a.z, a.rows, a.n_entries), grid, stream);
}

cudaError_t nr_learned_launch(const NrKernel& k, const cbn::NrLearnedArgs& la, int grid, cudaStream_t stream) {
  const cbn::NrArgs& a = la.a;
  return launch_with(k, &la, a.z, cbn::nr_learned_smem_bytes(a.n_full, a.z, a.rows, a.n_entries), grid, stream);
}

}  // namespace cbk
