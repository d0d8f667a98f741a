// The reference's file formats (declared in include/fdp_io.h).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fdp.h"
#include "fdp_io.h"

namespace {

std::string upper(std::string s) {
  for (char& ch : s) ch = (char)std::toupper((unsigned char)ch);
  return s;
}

// Strips '!' comments outside quotes.
std::string strip_comments(const std::string& t) {
  std::string o;
  char q = 0;
  bool comment = false;
  for (char ch : t) {
    if (comment) {
      if (ch == '\n') { comment = false; o += ch; }
      continue;
    }
    if (q) {
      if (ch == q) q = 0;
      o += ch;
    } else if (ch == '\'' || ch == '"') {
      q = ch;
      o += ch;
    } else if (ch == '!') {
      comment = true;
    } else {
      o += ch;
    }
  }
  return o;
}

// Body of namelist group `group` (between "&GROUP" and its terminating
// "/" or "&END"), or false when absent.
bool group_body(const std::string& text, const std::string& group, std::string& body) {
  const std::string t = strip_comments(text), U = upper(t), G = "&" + upper(group);
  size_t pos = 0;
  while ((pos = U.find(G, pos)) != std::string::npos) {
    const size_t after = pos + G.size();
    if (after < U.size() && (std::isalnum((unsigned char)U[after]) || U[after] == '_')) { pos = after; continue; }
    char q = 0;
    for (size_t i = after; i < t.size(); ++i) {
      const char ch = t[i];
      if (q) { if (ch == q) q = 0; continue; }
      if (ch == '\'' || ch == '"') { q = ch; continue; }
      if (ch == '/' || (ch == '&' && U.compare(i, 4, "&END") == 0)) {
        body = t.substr(after, i - after);
        return true;
      }
    }
    body = t.substr(after);
    return true;
  }
  return false;
}

}  // namespace

extern "C" {

int fdp_io_format_e(double v, int32_t w, int32_t d, char* out) {
  if (!out || w < 1 || d < 1 || d > 40) return FDP_ERR_ARG;
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
    if ((int)s.size() > w) s = v < 0 ? "-Inf" : "Inf";
  } else {
    const bool neg = std::signbit(v);
    std::string digits;
    int e10 = 0;
    if (v == 0.0) {
      digits.assign((size_t)d, '0');
    } else {
      // d significant digits, correctly rounded: D.DDDDDe+XX
      char buf[96];
      std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(v));
      const char* ep = std::strchr(buf, 'e');
      for (const char* c = buf; c < ep; ++c)
        if (std::isdigit((unsigned char)*c)) digits += *c;
      e10 = std::atoi(ep + 1) + 1;  // 0.DDDDDD x 10**e10
    }
    char ex[16];
    const int ae = std::abs(e10);
    if (ae <= 99) std::snprintf(ex, sizeof ex, "E%c%02d", e10 < 0 ? '-' : '+', ae);
    else if (ae <= 999) std::snprintf(ex, sizeof ex, "%c%03d", e10 < 0 ? '-' : '+', ae);
    else std::snprintf(ex, sizeof ex, "%c%d", e10 < 0 ? '-' : '+', ae);
    std::string body = "." + digits + ex;
    const std::string sign = neg ? "-" : "";
    // the optional leading zero is written when the field has room for it
    s = ((int)(sign.size() + body.size() + 1) <= w) ? sign + "0" + body : sign + body;
  }
  if ((int)s.size() > w) s.assign((size_t)w, '*');
  else s.insert(0, (size_t)(w - (int)s.size()), ' ');
  std::memcpy(out, s.c_str(), s.size() + 1);
  return FDP_OK;
}

int fdp_io_namelist_get(const char* text, const char* group, const char* name, char* out, size_t size) {
  if (!text || !group || !name || !out || size == 0) return FDP_ERR_ARG;
  std::string body;
  if (!group_body(text, group, body)) return FDP_ERR_ARG;
  const std::string N = upper(name);
  size_t i = 0;
  const size_t n = body.size();
  auto skip = [&]() {
    while (i < n && (std::isspace((unsigned char)body[i]) || body[i] == ',')) ++i;
  };
  while (true) {
    skip();
    if (i >= n) break;
    size_t a = i;
    while (i < n && (std::isalnum((unsigned char)body[i]) || body[i] == '_' || body[i] == '%')) ++i;
    const std::string key = upper(body.substr(a, i - a));
    while (i < n && std::isspace((unsigned char)body[i])) ++i;
    if (i >= n || body[i] != '=' || key.empty()) return FDP_ERR_ARG;  // malformed group
    ++i;
    while (i < n && std::isspace((unsigned char)body[i])) ++i;
    std::string val;
    if (i < n && (body[i] == '\'' || body[i] == '"')) {
      const char q = body[i++];
      while (i < n) {
        if (body[i] == q) {
          if (i + 1 < n && body[i + 1] == q) { val += q; i += 2; continue; }
          ++i;
          break;
        }
        val += body[i++];
      }
    } else {
      a = i;
      while (i < n && !std::isspace((unsigned char)body[i]) && body[i] != ',') ++i;
      val = body.substr(a, i - a);
    }
    if (key == N) {
      if (val.size() + 1 > size) return FDP_ERR_ARG;
      std::memcpy(out, val.c_str(), val.size() + 1);
      return FDP_OK;
    }
  }
  return FDP_ERR_ARG;
}

int fdp_io_read_record(const char* path, int64_t index, void* buf, int64_t capacity, int64_t* nbytes) {
  if (!path || index < 0 || !nbytes) return FDP_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return FDP_ERR_ARG;
  int64_t rec = 0, got = 0;
  int rc = FDP_ERR_ARG;
  while (true) {
    int32_t head;
    if (std::fread(&head, 4, 1, f) != 1) break;
    const int64_t len = head < 0 ? -(int64_t)head : head;
    const bool more = head < 0;  // a negative head marker: another subrecord follows
    if (rec == index) {
      if (buf && got + len > capacity) break;
      if (buf ? std::fread((char*)buf + got, 1, (size_t)len, f) != (size_t)len : std::fseek(f, len, SEEK_CUR) != 0) break;
      got += len;
    } else if (std::fseek(f, len, SEEK_CUR) != 0) {
      break;
    }
    int32_t tail;
    if (std::fread(&tail, 4, 1, f) != 1) break;
    if (!more) {
      if (rec == index) { *nbytes = got; rc = FDP_OK; break; }
      ++rec;
    }
  }
  std::fclose(f);
  return rc;
}

int fdp_io_append_record(const char* path, const void* buf, int64_t nbytes) {
  if (!path || (!buf && nbytes > 0) || nbytes < 0) return FDP_ERR_ARG;
  FILE* f = std::fopen(path, "ab");
  if (!f) return FDP_ERR_ARG;
  const int64_t kMax = 2147483639;  // gfortran's largest subrecord
  int64_t done = 0;
  bool ok = true, first = true;
  do {
    const int64_t len = std::min<int64_t>(nbytes - done, kMax);
    const bool more = done + len < nbytes;
    const int32_t head = (int32_t)(more ? -len : len);
    const int32_t tail = (int32_t)(first ? len : -len);
    ok = ok && std::fwrite(&head, 4, 1, f) == 1;
    ok = ok && (len == 0 || std::fwrite((const char*)buf + done, 1, (size_t)len, f) == (size_t)len);
    ok = ok && std::fwrite(&tail, 4, 1, f) == 1;
    done += len;
    first = false;
  } while (done < nbytes && ok);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? FDP_OK : FDP_ERR_ARG;
}

}  // extern "C"
