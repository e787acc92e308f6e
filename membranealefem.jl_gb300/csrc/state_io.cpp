// state_io.cpp -- the reference's state files and an asynchronous writer.
//
// run_analysis! writes the column-major xms (numnp x 3) and cps (numnp x ndf)
// matrices after every step with writedlm (src/Analysis.jl:75-78, the initial
// state at src/Input.jl:113-114), and prepare_input / restart read them back
// with readdlm (src/Input.jl:35-37, src/MembraneAleFem.jl:75-107).
//
// Format (DelimitedFiles' defaults): one matrix row per line, entries
// separated by one tab, '\n' line ends.  Each Float64 is printed as Julia's
// print(::Float64) does: the shortest decimal that reads back to the same
// double, in fixed notation when the decimal point falls within
// -4 < pt <= 6 digits of the first digit ("0.0001", "100000.0",
// "0.30000000000000004"), otherwise d.ddd e±X ("1.0e-5", "1.0e6",
// "-2.5e20"); "-0.0", "NaN", "Inf", "-Inf".  Reading accepts any run of tabs
// or spaces as a separator (readdlm's default) and checks the matrix shape.
//
// StateWriter lets a time loop write these files without waiting for them:
// the state is copied device -> pinned host on the handle's stream (ordered
// after the step that produced it), and a thread formats and writes the files
// once that copy has completed, while the GPU runs the next steps.

#include <cuda_runtime.h>

#include <cerrno>
#include <charconv>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mafem.h"
#include "mafem_internal.h"

namespace mafem {

void format_double(double x, std::string& out) {
  if (std::isnan(x)) {
    out += "NaN";
    return;
  }
  if (std::isinf(x)) {
    out += x > 0 ? "Inf" : "-Inf";
    return;
  }
  if (x == 0.0) {
    out += std::signbit(x) ? "-0.0" : "0.0";
    return;
  }
  // shortest round-trip digits, scientific: [-]d[.ddd]e[+-]XX
  char buf[64];
  const auto res = std::to_chars(buf, buf + sizeof buf - 1, x, std::chars_format::scientific);
  *res.ptr = '\0';  // to_chars does not terminate; atoi below reads up to the NUL
  const char* p = buf;
  const char* end = res.ptr;
  if (*p == '-') {
    out += '-';
    ++p;
  }
  char digits[24];
  int nd = 0;
  for (; p < end && *p != 'e'; ++p)
    if (*p != '.') digits[nd++] = *p;
  const int e = std::atoi(p + 1);  // x = 0.d1d2... * 10^(e+1)
  const int pt = e + 1;            // decimal point after pt digits
  if (-4 < pt && pt <= 6) {
    if (pt <= 0) {
      out += "0.";
      out.append((size_t)-pt, '0');
      out.append(digits, (size_t)nd);
    } else if (pt >= nd) {
      out.append(digits, (size_t)nd);
      out.append((size_t)(pt - nd), '0');
      out += ".0";
    } else {
      out.append(digits, (size_t)pt);
      out += '.';
      out.append(digits + pt, (size_t)(nd - pt));
    }
  } else {
    out += digits[0];
    out += '.';
    if (nd > 1)
      out.append(digits + 1, (size_t)(nd - 1));
    else
      out += '0';
    out += 'e';
    out += std::to_string(e);
  }
}

int writedlm(const char* path, const double* a, int64_t rows, int64_t cols, std::string& err) {
  std::string text;
  text.reserve((size_t)(rows * cols * 22 + rows));
  for (int64_t i = 0; i < rows; ++i) {
    for (int64_t j = 0; j < cols; ++j) {
      if (j) text += '\t';
      format_double(a[i + rows * j], text);
    }
    text += '\n';
  }
  FILE* f = std::fopen(path, "w");
  if (!f) {
    err = std::string("cannot open ") + path + " for writing: " + std::strerror(errno);
    return MAFEM_ERR_ARG;
  }
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  if (std::fclose(f) != 0 || !ok) {
    err = std::string("write error on ") + path;
    return MAFEM_ERR_ARG;
  }
  return MAFEM_OK;
}

int readdlm(const char* path, double* a, int64_t rows, int64_t cols, std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open ") + path + ": " + std::strerror(errno);
    return MAFEM_ERR_ARG;
  }
  std::string text;
  char chunk[1 << 16];
  size_t k;
  while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) text.append(chunk, k);
  std::fclose(f);
  const char* p = text.c_str();
  const char* const stop_all = p + text.size();
  int64_t i = 0;
  while (p < stop_all) {
    const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(stop_all - p)));
    const char* end = eol ? eol : stop_all;
    int64_t j = 0;
    const char* q = p;
    bool blank = true;
    while (true) {
      while (q < end && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
      if (q >= end) break;
      blank = false;
      if (i >= rows) {
        err = std::string(path) + ": more than " + std::to_string(rows) + " rows";
        return MAFEM_ERR_ARG;
      }
      // from_chars reads '.' as the decimal point whatever the process locale
      // (a host that set a ',' locale must still read these files); it takes
      // "Inf", "NaN" in any case, but no leading '+', which is skipped here
      const char* b = (*q == '+' && q + 1 < end && *(q + 1) != '-') ? q + 1 : q;
      double v = 0.0;
      const auto res = std::from_chars(b, end, v);
      const char* stop = res.ptr;
      if (res.ec == std::errc::result_out_of_range) {
        // beyond the double range: +-0 for a negative exponent, else +-Inf,
        // as Julia's parse gives
        const char* ex = b;
        while (ex < stop && *ex != 'e' && *ex != 'E') ++ex;
        const bool tiny = ex + 1 < stop && *(ex + 1) == '-';
        v = std::copysign(tiny ? 0.0 : HUGE_VAL, *b == '-' ? -1.0 : 1.0);
      } else if (res.ec != std::errc() || stop == b) {
        err = std::string(path) + ": not a number in row " + std::to_string(i + 1);
        return MAFEM_ERR_ARG;
      }
      if (stop < end && *stop != ' ' && *stop != '\t' && *stop != '\r') {
        err = std::string(path) + ": not a number in row " + std::to_string(i + 1);
        return MAFEM_ERR_ARG;
      }
      if (j >= cols) {
        err = std::string(path) + ": row " + std::to_string(i + 1) + " has more than " + std::to_string(cols) +
              " entries";
        return MAFEM_ERR_ARG;
      }
      a[i + rows * j] = v;
      ++j;
      q = stop;
    }
    if (!blank) {
      if (j != cols) {
        err = std::string(path) + ": row " + std::to_string(i + 1) + " has " + std::to_string(j) +
              " entries, expected " + std::to_string(cols);
        return MAFEM_ERR_ARG;
      }
      ++i;
    }
    p = eol ? eol + 1 : stop_all;
  }
  if (i != rows) {
    err = std::string(path) + ": " + std::to_string(i) + " rows, expected " + std::to_string(rows);
    return MAFEM_ERR_ARG;
  }
  return MAFEM_OK;
}

// ---------------------------------------------------------------------------

StateWriter::~StateWriter() {
  std::string ignored;
  flush(ignored);
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_job_.notify_all();
  if (th_.joinable()) th_.join();
  for (auto& s : slots_) {
    if (s.ev) cudaEventDestroy(s.ev);
    if (s.host) cudaFreeHost(s.host);
  }
}

int StateWriter::init(int numnp, int ndf, int depth, std::string& err) {
  numnp_ = numnp;
  ndf_ = ndf;
  cudaGetDevice(&device_);
  slots_.resize((size_t)depth);
  for (auto& s : slots_) {
    cudaError_t e = cudaMallocHost(&s.host, sizeof(double) * (size_t)numnp * (3 + ndf));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      err = std::string("state writer: ") + cudaGetErrorString(e);
      return MAFEM_ERR_CUDA;
    }
  }
  th_ = std::thread([this] { run(); });
  return MAFEM_OK;
}

int StateWriter::submit(const double* d_xms, const double* d_cps, cudaStream_t st, std::string xms_path,
                        std::string cps_path, std::string& err) {
  std::unique_lock<std::mutex> lk(mu_);
  int slot = -1;
  cv_free_.wait(lk, [&] {
    for (size_t s = 0; s < slots_.size(); ++s)
      if (!slots_[s].busy) {
        slot = (int)s;
        return true;
      }
    return false;
  });
  Slot& s = slots_[(size_t)slot];
  const size_t nx = (size_t)numnp_ * 3, nc = (size_t)numnp_ * ndf_;
  cudaError_t e = cudaMemcpyAsync(s.host, d_xms, sizeof(double) * nx, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s.host + nx, d_cps, sizeof(double) * nc, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaEventRecord(s.ev, st);
  if (e != cudaSuccess) {
    err = std::string("state writer copy: ") + cudaGetErrorString(e);
    return MAFEM_ERR_CUDA;
  }
  s.busy = true;
  s.xms_path = std::move(xms_path);
  s.cps_path = std::move(cps_path);
  queue_.push_back(slot);
  lk.unlock();
  cv_job_.notify_one();
  return MAFEM_OK;
}

int StateWriter::flush(std::string& err) {
  std::unique_lock<std::mutex> lk(mu_);
  cv_free_.wait(lk, [&] {
    for (const auto& s : slots_)
      if (s.busy) return false;
    return true;
  });
  const int rc = first_rc_;
  if (rc) err = first_err_;
  first_rc_ = MAFEM_OK;
  first_err_.clear();
  return rc;
}

void StateWriter::run() {
  cudaSetDevice(device_);
  while (true) {
    int slot;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_job_.wait(lk, [&] { return stop_ || !queue_.empty(); });
      if (queue_.empty()) return;
      slot = queue_.front();
      queue_.pop_front();
    }
    Slot& s = slots_[(size_t)slot];
    std::string err;
    int rc = MAFEM_OK;
    const cudaError_t e = cudaEventSynchronize(s.ev);
    if (e != cudaSuccess) {
      err = std::string("state writer: ") + cudaGetErrorString(e);
      rc = MAFEM_ERR_CUDA;
    }
    if (!rc) rc = writedlm(s.xms_path.c_str(), s.host, numnp_, 3, err);
    if (!rc) rc = writedlm(s.cps_path.c_str(), s.host + (size_t)numnp_ * 3, numnp_, ndf_, err);
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (rc && !first_rc_) {
        first_rc_ = rc;
        first_err_ = err;
      }
      s.busy = false;
    }
    cv_free_.notify_all();
  }
}

std::string state_file(const char* dir, int64_t t_id, const char* which) {
  std::string s(dir);
  s += "/t";
  s += std::to_string(t_id);
  s += '-';
  s += which;
  s += ".txt";
  return s;
}

}  // namespace mafem

using namespace mafem;

extern "C" int mafem_format_double(double x, char* buf, int32_t cap) {
  if (!buf || cap < 1) return MAFEM_ERR_ARG;
  std::string s;
  format_double(x, s);
  if ((int32_t)s.size() >= cap) return MAFEM_ERR_ARG;
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return (int)s.size();
}

extern "C" int mafem_writedlm(const char* path, const double* a, int64_t rows, int64_t cols) {
  if (!path || rows < 0 || cols < 0 || (!a && rows * cols > 0)) return MAFEM_ERR_ARG;
  std::string err;
  const int rc = writedlm(path, a, rows, cols, err);
  if (rc) set_global_error(err);
  return rc;
}

extern "C" int mafem_readdlm(const char* path, double* a, int64_t rows, int64_t cols) {
  if (!path || rows < 0 || cols < 0 || (!a && rows * cols > 0)) return MAFEM_ERR_ARG;
  std::string err;
  const int rc = readdlm(path, a, rows, cols, err);
  if (rc) set_global_error(err);
  return rc;
}
