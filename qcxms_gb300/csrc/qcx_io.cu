// Trajectory start files of a QCxMS ensemble, read on the host so that a
// batched driver can replace the one-process-per-trajectory fan-out.
//
// The production run writes, per trajectory n, TMPQCXMS/TMP.n/start.xyz (the
// structure, xyz format in Angstrom, written with mctc-io's write_structure)
// and TMPQCXMS/TMP.n/qcxms.start (wrstart, src/utility.f90:321-373):
//   line 1        the trajectory number, format (i4)
//   line 2        eimp (Eh), format (D22.14)
//   line 3        tadd (atomic time units), format (D22.14)
//   lines 4..     per atom vx vy vz velof, format (7D22.14) (4 fields used)
// rdstart (src/utility.f90:379-422) reads the same layout back.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qcxgpu.h"
#include "qcx_kernels.h"

namespace {

// Angstrom -> Bohr, src/xtb_mctc_convert.f90:24-25
constexpr double kAAtoAU = 1.0 / 0.52917726;

const char* const kSymbols[] = {"",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",
                                "Ne", "Na", "Mg", "Al", "Si", "P",  "S",  "Cl", "Ar"};

bool read_lines(const char* path, std::vector<std::string>& lines) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  std::string cur;
  int c;
  while ((c = std::fgetc(f)) != EOF) {
    if (c == '\n') {
      lines.push_back(cur);
      cur.clear();
    } else if (c != '\r') {
      cur.push_back((char)c);
    }
  }
  if (!cur.empty()) lines.push_back(cur);
  std::fclose(f);
  return true;
}

// one Fortran real in E or D exponent notation
bool parse_real(const std::string& tok, double* out) {
  std::string t = tok;
  for (char& ch : t)
    if (ch == 'D' || ch == 'd') ch = 'E';
  char* end = nullptr;
  *out = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && !t.empty();
}

// Fields of a fixed-width Fortran record: width characters each.
bool fixed_fields(const std::string& line, int width, int n, double* out) {
  for (int k = 0; k < n; ++k) {
    if ((int)line.size() < (k + 1) * width) return false;
    std::string f = line.substr((size_t)k * width, (size_t)width);
    size_t a = f.find_first_not_of(' '), b = f.find_last_not_of(' ');
    if (a == std::string::npos) return false;
    if (!parse_real(f.substr(a, b - a + 1), out + k)) return false;
  }
  return true;
}

std::vector<std::string> split(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j])) ++j;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

int symbol_to_z(const std::string& tok) {
  if (std::isdigit((unsigned char)tok[0])) {
    int z = std::atoi(tok.c_str());
    return (z >= 1 && z <= 18) ? z : -1;
  }
  std::string s;
  for (char ch : tok)
    if (std::isalpha((unsigned char)ch)) s.push_back(s.empty() ? (char)std::toupper(ch) : (char)std::tolower(ch));
  for (int z = 1; z <= 18; ++z)
    if (s == kSymbols[z]) return z;
  return -1;
}

// Fortran Dw.d edit descriptor: 0.<d digits>D<sign><2 digits>, right-justified
// in w characters; the mantissa digits are the value rounded to d significant
// digits (the round-to-nearest of printf's %.(d-1)E). A three-digit exponent
// drops the D (0.<digits><sign><3 digits>); a field too narrow is w asterisks.
std::string fortran_d(double x, int w, int d) {
  char buf[64];
  std::string out;
  if (x == 0.0) {
    out = "0." + std::string((size_t)d, '0') + "D+00";
  } else {
    std::snprintf(buf, sizeof(buf), "%.*E", d - 1, std::fabs(x));
    std::string m(buf);
    const size_t e = m.find('E');
    const int ex = std::atoi(m.c_str() + e + 1) + 1;
    std::string digits = m.substr(0, 1) + m.substr(2, e - 2);
    char tail[16];
    const int ax = ex < 0 ? -ex : ex;
    if (ax <= 99) std::snprintf(tail, sizeof(tail), "D%c%02d", ex < 0 ? '-' : '+', ax);
    else std::snprintf(tail, sizeof(tail), "%c%03d", ex < 0 ? '-' : '+', ax);
    out = std::string(x < 0 ? "-" : "") + "0." + digits + tail;
  }
  if ((int)out.size() > w) return std::string((size_t)w, '*');
  if ((int)out.size() < w) out = std::string((size_t)w - out.size(), ' ') + out;
  return out;
}

std::string fortran_d22_14(double x) { return fortran_d(x, 22, 14); }

// Fortran Iw: right-justified, w asterisks when the number does not fit
std::string fortran_i(long long v, int w) {
  char buf[32];
  std::snprintf(buf, sizeof(buf), "%lld", v);
  std::string s(buf);
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)w - s.size(), ' ') + s;
}

// Fortran Fw.d (gfortran prints the leading zero of |x| < 1 when it fits)
std::string fortran_f(double x, int w, int d) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%*.*f", w, d, x);
  std::string s(buf);
  if ((int)s.size() > w) {
    // without the optional leading zero, if that makes it fit
    size_t z = s.find("0.");
    if (z != std::string::npos && (z == 0 || s[z - 1] == '-' || s[z - 1] == ' ') && (int)s.size() - 1 <= w)
      s.erase(z, 1);
    if ((int)s.size() > w) return std::string((size_t)w, '*');
  }
  return s;
}

// gfortran's list-directed output of one REAL(8) item: a blank, then the item
// in 25 columns with 17 significant digits, 1PG25.17E3 style: F editing with
// 16 - e decimals and five trailing blanks for 0.1 <= |x| < 1e17 (e = the
// decimal exponent after rounding), else E editing with one digit before the
// point and a three-digit exponent. List-directed layout is processor
// dependent; this is the layout of gfortran, which the reference builds with.
std::string fortran_list_real(double x) {
  char buf[64];
  std::string body;
  if (x == 0.0) {
    body = std::string(std::signbit(x) ? "-" : "") + "0.0000000000000000     ";
  } else {
    std::snprintf(buf, sizeof(buf), "%.16e", x);
    std::string m(buf);
    const size_t p = m.find('e');
    const int ex = std::atoi(m.c_str() + p + 1);
    if (ex >= -1 && ex < 17) {
      std::snprintf(buf, sizeof(buf), "%.*f", 16 - ex, x);
      body = buf;
      if (16 - ex == 0) body += ".";
      body += "     ";
    } else {
      char tail[16];
      std::snprintf(tail, sizeof(tail), "E%c%03d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
      body = m.substr(0, p) + tail;
    }
  }
  if (body.size() < 25) body = std::string(25 - body.size(), ' ') + body;
  return " " + body;
}

// list-directed INTEGER item of gfortran: a blank and 11 columns
std::string fortran_list_int(long long v) {
  char buf[32];
  std::snprintf(buf, sizeof(buf), " %11lld", v);
  return buf;
}

}  // namespace

extern "C" {

int qcx_write_qmo(const char* tmp_path, const char* mspec_path, int nat, int nao, int ihomo, const double* emo,
                  const double* focc, const double* qmo) {
  if (nat < 1 || nao < 1 || !emo || !focc || !qmo) {
    qcx::set_last_error("qcx_write_qmo: invalid arguments (nat >= 1, nao >= 1, emo, focc and qmo)");
    return -1;
  }
  const double autoev = 27.21138505;  // src/xtb_mctc_convert.f90:27
  if (mspec_path) {
    // qcxms.Mspec.tbxtb: write(*) nao, ihomo; per orbital an empty record,
    // (i3,1x,f10.3) k and emo*autoev, (1x,f6.2) focc, (10(1x,f6.2)) the
    // populations in percent, ten to a line
    FILE* f = std::fopen(mspec_path, "w");
    if (!f) {
      qcx::set_last_error(std::string("qcx_write_qmo: cannot write ") + mspec_path);
      return -1;
    }
    std::fprintf(f, "%s%s\n", fortran_list_int(nao).c_str(), fortran_list_int(ihomo).c_str());
    for (int k = 0; k < nao; ++k) {
      std::fprintf(f, "\n%s %s\n %s\n", fortran_i(k + 1, 3).c_str(), fortran_f(emo[k] * autoev, 10, 3).c_str(),
                   fortran_f(focc[k], 6, 2).c_str());
      std::string line;
      for (int a = 0; a < nat; ++a) {
        line += " " + fortran_f(qmo[(size_t)k * nat + a] * 100.0, 6, 2);
        if (a % 10 == 9 || a == nat - 1) {
          std::fprintf(f, "%s\n", line.c_str());
          line.clear();
        }
      }
    }
    if (std::fclose(f) != 0) {
      qcx::set_last_error(std::string("qcx_write_qmo: write error on ") + mspec_path);
      return -1;
    }
  }
  if (tmp_path) {
    // tmp.mspec, list-directed throughout: nao, ihomo; per orbital emo*autoev,
    // focc and the nat populations, one item to a record
    FILE* f = std::fopen(tmp_path, "w");
    if (!f) {
      qcx::set_last_error(std::string("qcx_write_qmo: cannot write ") + tmp_path);
      return -1;
    }
    std::fprintf(f, "%s%s\n", fortran_list_int(nao).c_str(), fortran_list_int(ihomo).c_str());
    for (int k = 0; k < nao; ++k) {
      std::fprintf(f, "%s\n%s\n", fortran_list_real(emo[k] * autoev).c_str(), fortran_list_real(focc[k]).c_str());
      for (int a = 0; a < nat; ++a) std::fprintf(f, "%s\n", fortran_list_real(qmo[(size_t)k * nat + a]).c_str());
    }
    if (std::fclose(f) != 0) {
      qcx::set_last_error(std::string("qcx_write_qmo: write error on ") + tmp_path);
      return -1;
    }
  }
  return 0;
}


int qcx_write_start(const char* path, int itrj, int nat, double eimp, double tadd, const double* vel,
                    const double* velof) {
  if (!path || nat < 1 || !vel || !velof || itrj < 0 || itrj > 9999) {
    qcx::set_last_error("qcx_write_start: invalid arguments (0 <= itrj <= 9999, nat >= 1, vel and velof)");
    return -1;
  }
  FILE* f = std::fopen(path, "w");
  if (!f) {
    qcx::set_last_error(std::string("qcx_write_start: cannot write ") + path);
    return -1;
  }
  std::fprintf(f, "%4d\n%s\n%s\n", itrj, fortran_d22_14(eimp).c_str(), fortran_d22_14(tadd).c_str());
  for (int a = 0; a < nat; ++a)
    std::fprintf(f, "%s%s%s%s\n", fortran_d22_14(vel[3 * a]).c_str(), fortran_d22_14(vel[3 * a + 1]).c_str(),
                 fortran_d22_14(vel[3 * a + 2]).c_str(), fortran_d22_14(velof[a]).c_str());
  const bool ok = std::fclose(f) == 0;
  if (!ok) qcx::set_last_error(std::string("qcx_write_start: write error on ") + path);
  return ok ? 0 : -1;
}

int qcx_write_gs(const char* path, int nmax, int nat, int nrec, const double* xyz, const double* vel) {
  if (!path || nat < 1 || nrec < 0 || (nrec > 0 && (!xyz || !vel))) {
    qcx::set_last_error("qcx_write_gs: invalid arguments (nat >= 1, nrec >= 0, xyz and vel)");
    return -1;
  }
  FILE* f = std::fopen(path, "w");
  if (!f) {
    qcx::set_last_error(std::string("qcx_write_gs: cannot write ") + path);
    return -1;
  }
  // write(io_GS,*) nmax: list-directed, a blank and the integer in 11 columns
  std::fprintf(f, " %11d\n", nmax);
  for (long long r = 0; r < nrec; ++r)
    for (int a = 0; a < nat; ++a) {
      const double* x = xyz + (r * nat + a) * 3;
      const double* v = vel + (r * nat + a) * 3;
      std::string line;
      for (int k = 0; k < 3; ++k) line += fortran_d(x[k], 16, 8);
      for (int k = 0; k < 3; ++k) line += fortran_d(v[k], 16, 8);
      std::fprintf(f, "%s\n", line.c_str());
    }
  const bool ok = std::fclose(f) == 0;
  if (!ok) qcx::set_last_error(std::string("qcx_write_gs: write error on ") + path);
  return ok ? 0 : -1;
}

int qcx_format_res(int cid, double fragchrg3, int mchrg, int itrj, int icoll, int isec, int ifrag, int nel,
                   const int32_t* z, const int32_t* count, char* line, int len) {
  if (!line || len < 1 || nel < 0 || nel > 20 || (nel > 0 && (!z || !count))) {
    qcx::set_last_error("qcx_format_res: invalid arguments (0 <= nel <= 20, z and count, an output buffer)");
    return -1;
  }
  // items in the order of the write statement; the edit descriptors
  // F10.7, i3, 2i5, 2i2, 2x, i3, 2x, 20(i4, i3) take them in turn
  std::vector<long long> items;
  items.push_back(mchrg);
  items.push_back(itrj);
  if (cid) items.push_back(icoll);
  items.push_back(isec);
  items.push_back(ifrag);
  items.push_back(nel);
  for (int m = 0; m < nel; ++m) {
    items.push_back(z[m]);
    items.push_back(count[m]);
  }
  static const int kWidth[] = {3, 5, 5, 2, 2, 3};  // i3, 2i5, 2i2, 2x, i3
  std::string out = fortran_f(fragchrg3, 10, 7);
  for (size_t k = 0; k < items.size(); ++k) {
    if (k == 5) out += "  ";                 // the 2x before i3
    if (k == 6) out += "  ";                 // the 2x after it
    const int w = k < 6 ? kWidth[k] : ((k - 6) % 2 == 0 ? 4 : 3);
    out += fortran_i(items[k], w);
  }
  if ((int)out.size() + 1 > len) {
    qcx::set_last_error("qcx_format_res: output buffer too small");
    return -1;
  }
  std::memcpy(line, out.c_str(), out.size() + 1);
  return (int)out.size();
}

int qcx_read_xyz(const char* path, int max_nat, int32_t* nat, int32_t* num, double* xyz) {
  std::vector<std::string> lines;
  if (!path || !nat || max_nat < 0 || !read_lines(path, lines)) {
    qcx::set_last_error(std::string("qcx_read_xyz: cannot read ") + (path ? path : "(null)"));
    return -1;
  }
  std::vector<std::string> head = lines.empty() ? std::vector<std::string>() : split(lines[0]);
  int n = head.size() == 1 ? std::atoi(head[0].c_str()) : -1;
  if (n < 1 || (int)lines.size() < n + 2) {
    qcx::set_last_error(std::string("qcx_read_xyz: not an xyz file: ") + path);
    return -1;
  }
  *nat = n;
  if (!num && !xyz) return 0;  // size query
  if (n > max_nat) {
    qcx::set_last_error("qcx_read_xyz: more atoms than max_nat");
    return -1;
  }
  for (int a = 0; a < n; ++a) {
    std::vector<std::string> t = split(lines[2 + a]);
    double v[3];
    int z = t.size() >= 4 ? symbol_to_z(t[0]) : -1;
    if (z < 1 || !parse_real(t[1], v) || !parse_real(t[2], v + 1) || !parse_real(t[3], v + 2)) {
      qcx::set_last_error(std::string("qcx_read_xyz: bad atom line (elements 1..18) in ") + path);
      return -1;
    }
    if (num) num[a] = z;
    if (xyz)
      for (int d = 0; d < 3; ++d) xyz[3 * a + d] = v[d] * kAAtoAU;
  }
  return 0;
}

int qcx_read_start(const char* path, int nat, int32_t* itrj, double* eimp, double* tadd, double* vel,
                   double* velof) {
  std::vector<std::string> lines;
  if (!path || nat < 1 || !read_lines(path, lines)) {
    qcx::set_last_error(std::string("qcx_read_start: cannot read ") + (path ? path : "(null)"));
    return -1;
  }
  if ((int)lines.size() < 3 + nat) {
    qcx::set_last_error(std::string("qcx_read_start: fewer lines than 3 + nat in ") + path);
    return -1;
  }
  std::vector<std::string> t = split(lines[0]);
  double e, ta;
  if (t.size() != 1 || !fixed_fields(lines[1], 22, 1, &e) || !fixed_fields(lines[2], 22, 1, &ta)) {
    qcx::set_last_error(std::string("qcx_read_start: bad header in ") + path);
    return -1;
  }
  if (itrj) *itrj = std::atoi(t[0].c_str());
  if (eimp) *eimp = e;
  if (tadd) *tadd = ta;
  for (int a = 0; a < nat; ++a) {
    double v[4];
    if (!fixed_fields(lines[3 + a], 22, 4, v)) {
      qcx::set_last_error(std::string("qcx_read_start: bad velocity record in ") + path);
      return -1;
    }
    if (vel)
      for (int d = 0; d < 3; ++d) vel[3 * a + d] = v[d];
    if (velof) velof[a] = v[3];
  }
  return 0;
}

}  // extern "C"
