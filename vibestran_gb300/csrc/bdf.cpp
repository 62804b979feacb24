// vibestran_gb300/csrc/bdf.cpp — native reader of the BDF decks of the SOL 101
// CHEXA8 path.
//
// Reads the deck subset that path consumes — GRID, CHEXA, PSOLID, MAT1, SPC1,
// FORCE and PARAM in the bulk data; SOL, SUBCASE, LOAD, SPC, MPC and
// TEMP(LOAD) in the case control — with the card assembly and number rules of
// BdfParser::parse_stream (src/io/bdf_parser.cpp:95-700):
//   * CR-stripped lines; SOL / BEGIN BULK / ENDDATA markers; '$' comments;
//   * free-field lines (any comma), small-field (8-column) and large-field
//     (16-column, "GRID*" / "*GRID") lines;
//   * '+', bare '*' and blank-label continuation lines, their fields 1-8
//     appended to the card;
//   * Nastran numbers: implicit exponents ("1.5+3", "2.-4") and D exponents.
// Cards the reference parses but this path cannot represent (other element
// types, rigid elements) make the deck unusable and are reported by name, as
// are loads and SPCs outside the path when the chosen subcase selects their
// set; cards the reference does not know are ignored and listed, as there.
//
// Throughput: the file is read in one piece and indexed by lines; the bulk
// section is cut into chunks at card starts and parsed by host threads into
// typed per-chunk records (string_view fields, from_chars numbers, no
// allocation per field), which are concatenated in file order.

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <string_view>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/vsgb.h"

namespace {

using sv = std::string_view;

struct ParseFail {
  long long line;  // 1-based line of the card (0: no line)
  std::string msg;
};

inline bool is_blank(char c) { return c == ' ' || c == '\t'; }
// std::isspace in the C locale
inline bool is_space(char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }
inline char up(char c) { return (c >= 'a' && c <= 'z') ? static_cast<char>(c - 32) : c; }

sv trim_blank(sv s) {  // find_first_not_of / find_last_not_of(" \t")
  size_t b = 0, e = s.size();
  while (b < e && is_blank(s[b])) ++b;
  while (e > b && is_blank(s[e - 1])) --e;
  return s.substr(b, e - b);
}

bool starts_ci(sv s, sv prefix) {
  if (s.size() < prefix.size()) return false;
  for (size_t i = 0; i < prefix.size(); ++i)
    if (up(s[i]) != prefix[i]) return false;
  return true;
}

std::string upper(sv s) {
  std::string o(s);
  for (char& c : o) c = up(c);
  return o;
}

// ── numbers (BdfParser::parse_double / parse_int, bdf_parser.cpp:780-818) ──

double parse_double(sv s, long long line) {
  if (s.empty()) return 0.0;
  // D exponent -> E; first +/- after position 0 not preceded by E -> "E+"/"E-"
  char small[64];
  std::string big;
  char* b = small;
  const size_t cap = s.size() + 2;
  if (cap > sizeof(small)) {
    big.resize(cap);
    b = big.data();
  }
  size_t n = 0;
  bool inserted = false;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (c == 'D' || c == 'd') c = 'E';
    if (!inserted && i > 0 && (c == '+' || c == '-') && up(b[n - 1]) != 'E') {
      b[n++] = 'E';
      inserted = true;
    }
    b[n++] = c;
  }
  b[n] = '\0';
  // fast path: plain decimal (from_chars takes no leading '+')
  const char* p = b;
  const char* end = b + n;
  if (*p == '+' && p + 1 < end && *(p + 1) != '-' && *(p + 1) != '+') ++p;
  double v = 0.0;
  const auto r = std::from_chars(p, end, v, std::chars_format::general);
  if (r.ec == std::errc()) return v;
  // anything else (hex, inf, out of range): strtod, failing as std::stod does
  errno = 0;
  char* stop = nullptr;
  v = std::strtod(b, &stop);
  if (stop == b || errno == ERANGE)
    throw ParseFail{line, "cannot parse double: '" + std::string(s) + "'"};
  return v;
}

int parse_int(sv s, long long line) {
  if (s.empty()) return 0;
  const char* p = s.data();
  const char* end = p + s.size();
  if (*p == '+' && p + 1 < end && *(p + 1) != '-' && *(p + 1) != '+') ++p;
  long long v = 0;
  const auto r = std::from_chars(p, end, v);  // leading digits, as std::stoi
  if (r.ec != std::errc() || v < INT_MIN || v > INT_MAX)
    throw ParseFail{line, "cannot parse int: '" + std::string(s) + "'"};
  return static_cast<int>(v);
}

// std::stoi of a case-control value: leading whitespace, then digits.
bool case_int(sv s, int* out) {
  size_t i = 0;
  while (i < s.size() && is_space(s[i])) ++i;
  try {
    *out = parse_int(s.substr(i), 0);
    return true;
  } catch (const ParseFail&) {
    return false;
  }
}

}  // namespace

// ── records ────────────────────────────────────────────────────────────────

struct vsgb_bdf {
  struct Grid {
    int id, cp, cd;
    double x[3];
    long long line;
  };
  struct Hexa {
    int eid, pid;
    int g[8];
    long long line;
  };
  struct Mat1 {
    int mid;
    double E, nu;
    long long line;
  };
  struct Psolid {
    int pid, mid, isop;  // VSGB_EAS / VSGB_SRI
    long long line;
  };
  struct Spc1 {
    int sid, mask, node;
    long long line;
  };
  struct Force {
    int sid, node, cid;
    double scale, dir[3];
    long long line;
  };
  // A card of the reference's set that this path cannot represent; sid is
  // its load / SPC set where it has one (-1: always in the model).
  struct Outside {
    std::string kw;
    int sid;
    long long line;
  };
  struct Chunk {
    std::vector<Grid> grids;
    std::vector<Hexa> hexas;
    std::vector<Mat1> mats;
    std::vector<Psolid> props;
    std::vector<Spc1> spcs;
    std::vector<Force> forces;
    std::vector<Outside> outside;
    std::set<std::string> ignored;  // keywords the reference does not parse either
    long long cards = 0;
    bool failed = false;
    ParseFail fail;
  };
  struct Subcase {
    int id = 1, load = 0, spc = 0, mpc = 0, temp = 0;
  };

  // deck
  int sol = 0;
  std::vector<Subcase> subcases;
  std::set<std::string> ignored_case;
  long long lines = 0, cards = 0;
  double read_ms = 0.0, parse_ms = 0.0, lines_ms = 0.0, cards_ms = 0.0, mesh_ms = 0.0;
  int threads = 1;
  Chunk all;  // records of every chunk, in file order

  // model (nodes sorted by id, duplicates: last card wins as a map insert)
  std::vector<int> node_ids;
  std::vector<double> xyz;
  std::vector<int> elem_ids, conn, form;
  std::vector<double> E, nu;
  std::string model_error;  // why the mesh cannot be formed (empty: it can)
  std::string warnings;
  std::string last_error;   // of the last failed call on this handle
};

namespace {

using Bdf = vsgb_bdf;

// Lines of text[a, b) (CR stripped), as getline sees them; a is a line start.
void split_range(sv text, size_t a, size_t b, std::vector<sv>& out) {
  size_t pos = a;
  while (pos < b) {
    const void* nl = std::memchr(text.data() + pos, '\n', text.size() - pos);
    const size_t e = nl ? static_cast<size_t>(static_cast<const char*>(nl) - text.data())
                        : text.size();
    sv l = text.substr(pos, e - pos);
    if (!l.empty() && l.back() == '\r') l.remove_suffix(1);
    out.push_back(l);
    pos = e + 1;
  }
}

// All lines, split by up to T threads over byte ranges that start at lines.
std::vector<sv> split_lines(sv text, int T) {
  std::vector<sv> out;
  if (T <= 1 || text.size() < (1u << 22)) {
    out.reserve(text.size() / 40 + 16);
    split_range(text, 0, text.size(), out);
    return out;
  }
  std::vector<size_t> st(static_cast<size_t>(T) + 1, text.size());
  st[0] = 0;
  for (int k = 1; k < T; ++k) {
    size_t s = text.size() * static_cast<size_t>(k) / static_cast<size_t>(T);
    s = std::max(s, st[static_cast<size_t>(k) - 1]);
    const void* nl = s < text.size() ? std::memchr(text.data() + s, '\n', text.size() - s) : nullptr;
    st[static_cast<size_t>(k)] =
        nl ? static_cast<size_t>(static_cast<const char*>(nl) - text.data()) + 1 : text.size();
  }
  std::vector<std::vector<sv>> parts(static_cast<size_t>(T));
  std::vector<std::thread> pool;
  for (int k = 0; k < T; ++k)
    pool.emplace_back([&, k] {
      auto& v = parts[static_cast<size_t>(k)];
      v.reserve((st[static_cast<size_t>(k) + 1] - st[static_cast<size_t>(k)]) / 40 + 16);
      split_range(text, st[static_cast<size_t>(k)], st[static_cast<size_t>(k) + 1], v);
    });
  for (auto& t : pool) t.join();
  size_t n = 0;
  for (const auto& v : parts) n += v.size();
  out.reserve(n);
  for (const auto& v : parts) out.insert(out.end(), v.begin(), v.end());
  return out;
}

int thread_count(int threads) {
  int T = threads;
  if (T <= 0) T = static_cast<int>(std::thread::hardware_concurrency());
  return T < 1 ? 1 : T;
}

sv lead_trimmed(sv l) {
  size_t f = 0;
  while (f < l.size() && is_blank(l[f])) ++f;
  return l.substr(f);
}

// ── case control (bdf_parser.cpp:110-409) ─────────────────────────────────

void parse_case_control(Bdf& d, const std::vector<sv>& lines, size_t begin_bulk) {
  Bdf::Subcase global, cur;
  bool in_sc = false, global_entries = false;
  auto value_after_eq = [](const std::string& kw, int* out) {
    const size_t eq = kw.find('=');
    return eq != std::string::npos && case_int(sv(kw).substr(eq + 1), out);
  };
  for (size_t i = 0; i < begin_bulk; ++i) {
    std::string u = upper(lines[i]);
    const size_t dlr = u.find('$');
    if (dlr != std::string::npos) u.resize(dlr);
    while (!u.empty() && is_space(u.back())) u.pop_back();
    const size_t first = u.find_first_not_of(" \t");
    if (first == std::string::npos) continue;
    const std::string kw = u.substr(first);
    Bdf::Subcase& sc = in_sc ? cur : global;
    bool entry = true;
    int v = 0;
    if (kw.rfind("SUBCASE", 0) == 0) {
      if (in_sc) d.subcases.push_back(cur);
      cur = global;
      cur.id = 1;
      in_sc = true;
      entry = false;
      const size_t eq = kw.find('=');
      if (eq != std::string::npos) {
        if (case_int(sv(kw).substr(eq + 1), &v)) cur.id = v;
      } else {
        const size_t sp = kw.find(' ');
        if (sp != std::string::npos && case_int(sv(kw).substr(sp + 1), &v)) cur.id = v;
      }
    } else if (kw.rfind("LOAD", 0) == 0) {
      if (value_after_eq(kw, &v)) sc.load = v;
    } else if (kw.rfind("MPC", 0) == 0 && kw.find('=') != std::string::npos &&
               kw.rfind("MPCADD", 0) != 0) {
      if (value_after_eq(kw, &v)) sc.mpc = v;
    } else if (kw.rfind("SPC", 0) == 0 && kw.rfind("SPCADD", 0) != 0) {
      if (value_after_eq(kw, &v)) sc.spc = v;
    } else if (kw.rfind("TEMP(LOAD)", 0) == 0 || kw.rfind("TEMPERATURE(LOAD)", 0) == 0) {
      if (value_after_eq(kw, &v)) sc.temp = v;
    } else if (kw == "CEND" || kw == "SOL" || kw.rfind("SOL ", 0) == 0 ||
               kw.rfind("BEGIN BULK", 0) == 0 || kw.rfind("BEGIN  BULK", 0) == 0) {
      entry = false;
    } else if (kw.rfind("LABEL", 0) == 0 || kw.rfind("DISPLACEMENT", 0) == 0 ||
               kw.rfind("STRESS", 0) == 0 || kw.rfind("STRAIN", 0) == 0 ||
               kw.rfind("METHOD", 0) == 0 || kw.rfind("EIGENVECTOR", 0) == 0 ||
               kw.rfind("VECTOR", 0) == 0 || kw.rfind("TEMP", 0) == 0 ||
               kw.rfind("TITLE", 0) == 0 || kw.rfind("SUBTITLE", 0) == 0 ||
               kw.rfind("ECHO", 0) == 0) {
      // output requests and titles: no effect on the solution
      const size_t eq = kw.find('=');
      if (eq != std::string::npos && trim_blank(sv(kw).substr(eq + 1)).rfind("NONE", 0) == 0)
        entry = false;
    } else {
      entry = false;
      const size_t end = kw.find_first_of(" =(,\t");
      d.ignored_case.insert(kw.substr(0, end));
    }
    if (entry && !in_sc) global_entries = true;
  }
  if (in_sc) d.subcases.push_back(cur);
  if (d.subcases.empty()) {
    // no SUBCASE: the global entries form subcase 1, or LOAD = SPC = 1
    if (global_entries) {
      d.subcases.push_back(global);
    } else {
      Bdf::Subcase s;
      s.load = s.spc = 1;
      d.subcases.push_back(s);
    }
  }
}

// SOL, BEGIN BULK and ENDDATA markers (bdf_parser.cpp:110-144): returns the
// first bulk line and the ENDDATA line (lines.size() when absent).
void find_markers(Bdf& d, const std::vector<sv>& lines, size_t* begin, size_t* end) {
  long long begin_bulk = -1;
  size_t enddata = lines.size();
  for (size_t i = 0; i < lines.size(); ++i) {
    const sv k = lead_trimmed(lines[i]);
    if (k.empty()) continue;
    const char c = up(k[0]);
    if (c != 'B' && c != 'E' && c != 'S') continue;
    if (starts_ci(k, "BEGIN BULK") || starts_ci(k, "BEGIN  BULK")) {
      begin_bulk = static_cast<long long>(i) + 1;
    } else if (starts_ci(k, "ENDDATA")) {
      enddata = i;
      break;
    } else if (begin_bulk == -1 && starts_ci(k, "SOL ")) {
      int v = 0;
      if (case_int(trim_blank(k.substr(4)), &v) && (v == 101 || v == 103)) d.sol = v;
    }
  }
  *begin = begin_bulk < 0 ? 0 : static_cast<size_t>(begin_bulk);
  *end = enddata;
}

// ── bulk data: logical cards (bdf_parser.cpp:411-541) ─────────────────────

bool is_comment_line(sv l) {
  size_t f = 0;
  while (f < l.size() && is_blank(l[f])) ++f;
  return f == l.size() || l[f] == '$';
}

bool is_continuation(sv l) {
  if (l.empty()) return false;
  const char c0 = l[0];
  if (c0 == '+') return true;
  const size_t kend = std::min<size_t>(l.size(), 8);
  if (c0 == '*') {
    // a bare '*' in columns 1-8 continues a large-field card; "*GRID" starts one
    for (size_t i = 1; i < kend; ++i)
      if (!is_space(l[i])) return false;
    return true;
  }
  if (is_space(c0)) {
    // blank label: columns 1-8 blank, data after them
    for (size_t i = 0; i < kend; ++i)
      if (!is_space(l[i])) return false;
    for (size_t i = kend; i < l.size(); ++i)
      if (!is_space(l[i])) return true;
  }
  return false;
}

void split_fixed(sv l, int width, int nfields, std::vector<sv>& f) {
  auto get = [&](size_t start, size_t w) -> sv {
    if (start >= l.size()) return sv();
    return trim_blank(l.substr(start, std::min(w, l.size() - start)));
  };
  f.push_back(get(0, 8));
  for (int i = 0; i < nfields; ++i) f.push_back(get(8 + static_cast<size_t>(i) * width, width));
}

void split_free(sv l, std::vector<sv>& f) {
  const size_t dlr = l.find('$');
  if (dlr != sv::npos) l = l.substr(0, dlr);
  const size_t first = f.size();
  size_t pos = 0;
  // std::getline(ss, tok, ','): a trailing comma yields no empty token
  while (pos < l.size()) {
    const size_t c = l.find(',', pos);
    const size_t e = c == sv::npos ? l.size() : c;
    f.push_back(trim_blank(l.substr(pos, e - pos)));
    pos = e + 1;
  }
  // a 10th field starting with '+' or '*' is a continuation label
  if (f.size() - first >= 10) {
    const sv f9 = f[first + 9];
    if (!f9.empty() && (f9[0] == '+' || f9[0] == '*'))
      f.erase(f.begin() + static_cast<long>(first + 9));
  }
}

// Fields of one physical line (keyword / label first).
void split_line(sv l, std::vector<sv>& f) {
  const bool free = l.find(',') != sv::npos;
  bool large = !l.empty() && l[0] == '*';
  if (!large && !free) {
    const size_t kend = std::min<size_t>(l.size(), 8);
    size_t last = kend;
    while (last > 0 && is_blank(l[last - 1])) --last;
    if (last > 0 && l[last - 1] == '*') large = true;
  }
  if (free) {
    split_free(l, f);
    // a trailing field starting with '+' marks a continuation
    if (!f.empty() && !f.back().empty() && f.back()[0] == '+') f.pop_back();
  } else if (large) {
    split_fixed(l, 16, 4, f);
  } else {
    split_fixed(l, 8, 8, f);
  }
}

// Keyword: upper case, leading '*' and trailing '*' / blanks removed.
std::string card_keyword(sv f0) {
  std::string kw = upper(f0);
  if (!kw.empty() && kw[0] == '*') kw.erase(0, 1);
  while (!kw.empty() && (kw.back() == '*' || is_space(kw.back()))) kw.pop_back();
  return kw;
}

// Bulk cards the reference parses (bdf_parser.cpp:555-662) that this path
// does not: elements and rigid elements are always in the model; loads, SPCs
// and MPCs only when the subcase selects their set (field 1).
enum class Kind { Path, Ignored, Element, SetCard, Harmless };

Kind classify(const std::string& kw) {
  static const std::unordered_map<std::string, Kind> k = {
      {"GRID", Kind::Path}, {"CHEXA", Kind::Path}, {"PSOLID", Kind::Path},
      {"MAT1", Kind::Path}, {"SPC1", Kind::Path}, {"FORCE", Kind::Path},
      {"PARAM", Kind::Path},
      {"CQUAD4", Kind::Element}, {"CTRIA3", Kind::Element}, {"CTETRA", Kind::Element},
      {"CPENTA", Kind::Element}, {"CBAR", Kind::Element}, {"CBEAM", Kind::Element},
      {"CBUSH", Kind::Element}, {"CELAS1", Kind::Element}, {"CELAS2", Kind::Element},
      {"CMASS1", Kind::Element}, {"CMASS2", Kind::Element}, {"RBE2", Kind::Element},
      {"RBE3", Kind::Element},
      {"MOMENT", Kind::SetCard}, {"GRAV", Kind::SetCard},
      {"ACCEL", Kind::SetCard}, {"ACCEL1", Kind::SetCard}, {"PLOAD", Kind::SetCard},
      {"PLOAD1", Kind::SetCard}, {"PLOAD2", Kind::SetCard}, {"PLOAD4", Kind::SetCard},
      {"SPC", Kind::SetCard},
      // materials / properties (used only through an element's PID), coordinate
      // systems (used only through CP / CD / CID, refused below), SOL 103 data,
      // MPCs (used only through an MPC set, refused below)
      {"MAT2", Kind::Harmless}, {"MAT3", Kind::Harmless}, {"MAT4", Kind::Harmless},
      {"MAT5", Kind::Harmless}, {"MAT6", Kind::Harmless}, {"MAT8", Kind::Harmless},
      {"PSHELL", Kind::Harmless}, {"PBAR", Kind::Harmless}, {"PBARL", Kind::Harmless},
      {"PBEAM", Kind::Harmless}, {"PBUSH", Kind::Harmless}, {"PELAS", Kind::Harmless},
      {"PMASS", Kind::Harmless}, {"CORD2R", Kind::Harmless}, {"CORD2C", Kind::Harmless},
      {"CORD2S", Kind::Harmless}, {"CORD1R", Kind::Harmless}, {"CORD1C", Kind::Harmless},
      {"EIGRL", Kind::Harmless}, {"MPC", Kind::Harmless}, {"MPCADD", Kind::Harmless},
      // nodal / default temperatures of the subcase's temperature set
      // (TEMPERATURE(LOAD), else its LOAD set: linear_static.cpp:82-100)
      {"TEMP", Kind::SetCard}, {"TEMPD", Kind::SetCard},
  };
  const auto it = k.find(kw);
  return it == k.end() ? Kind::Ignored : it->second;
}

// ── card processors (bdf_parser.cpp:1091-1306, 1473-1494, 1663-1675, 1958-1995) ──

void process_card(Bdf::Chunk& out, const std::string& kw, const std::vector<sv>& f,
                  long long line) {
  auto fld = [&](size_t i) -> sv { return i < f.size() ? f[i] : sv(); };
  if (kw == "GRID") {
    // GRID, ID, CP, X1, X2, X3, CD
    Bdf::Grid g;
    g.id = parse_int(fld(1), line);
    g.cp = fld(2).empty() ? 0 : parse_int(fld(2), line);
    for (int k = 0; k < 3; ++k) g.x[k] = parse_double(fld(3 + k), line);
    g.cd = fld(6).empty() ? 0 : parse_int(fld(6), line);
    g.line = line;
    out.grids.push_back(g);
  } else if (kw == "CHEXA") {
    // CHEXA, EID, PID, G1..G8 (blank slots skipped)
    Bdf::Hexa h;
    h.eid = parse_int(fld(1), line);
    h.pid = parse_int(fld(2), line);
    int cnt = 0;
    for (size_t i = 3; i < f.size(); ++i) {
      if (f[i].empty()) continue;
      const int g = parse_int(f[i], line);
      if (cnt < 8) h.g[cnt] = g;
      ++cnt;
    }
    if (cnt > 8)
      throw ParseFail{line, "CHEXA has " + std::to_string(cnt) +
                                " nodes; CHEXA20 is not yet supported"};
    if (cnt < 8)
      throw ParseFail{line, "CHEXA has " + std::to_string(cnt) + " nodes; expected 8"};
    h.line = line;
    out.hexas.push_back(h);
  } else if (kw == "MAT1") {
    // MAT1, MID, E, G, NU, RHO, A, TREF (all parsed, as the reference does)
    Bdf::Mat1 m;
    m.mid = parse_int(fld(1), line);
    m.E = parse_double(fld(2), line);
    for (size_t i : {3u, 5u, 6u, 7u})
      if (!fld(i).empty()) (void)parse_double(fld(i), line);
    m.nu = fld(4).empty() ? 0.0 : parse_double(fld(4), line);
    m.line = line;
    out.mats.push_back(m);
  } else if (kw == "PSOLID") {
    // PSOLID, PID, MID, CORDM, IN, STRESS, ISOP: ISOP "SRI" / "EAS"
    Bdf::Psolid p;
    p.pid = parse_int(fld(1), line);
    p.mid = parse_int(fld(2), line);
    if (!fld(3).empty()) (void)parse_int(fld(3), line);
    p.isop = VSGB_EAS;
    const std::string isop = upper(fld(6));
    if (isop == "SRI") p.isop = VSGB_SRI;
    p.line = line;
    out.props.push_back(p);
  } else if (kw == "SPC1") {
    // SPC1, SID, C, G1, G2, ... with "G1 THRU Gn"
    const int sid = parse_int(fld(1), line);
    int c = parse_int(fld(2), line), mask = 0;
    while (c > 0) {  // DofSet::from_int (include/core/types.hpp:114-124)
      const int digit = c % 10;
      if (digit >= 1 && digit <= 6) mask |= 1 << (digit - 1);
      c /= 10;
    }
    std::vector<int> nodes;
    bool thru = false;
    int start = 0;
    for (size_t i = 3; i < f.size(); ++i) {
      if (f[i].empty()) continue;
      if (upper(f[i]) == "THRU") {
        thru = true;
        if (!nodes.empty()) nodes.pop_back();
      } else if (thru) {
        const int last = parse_int(f[i], line);
        if (static_cast<long long>(last) - start > 100000000LL)
          throw ParseFail{line, "SPC1 THRU range longer than 1e8 grids"};
        for (long long nid = start; nid <= last; ++nid) nodes.push_back(static_cast<int>(nid));
        thru = false;
      } else {
        start = parse_int(f[i], line);
        nodes.push_back(start);
      }
    }
    for (int nid : nodes) out.spcs.push_back({sid, mask, nid, line});
  } else if (kw == "FORCE") {
    // FORCE, SID, G, CID, F, N1, N2, N3
    Bdf::Force fo;
    fo.sid = parse_int(fld(1), line);
    fo.node = parse_int(fld(2), line);
    fo.cid = fld(3).empty() ? 0 : parse_int(fld(3), line);
    fo.scale = parse_double(fld(4), line);
    for (int k = 0; k < 3; ++k) fo.dir[k] = parse_double(fld(5 + k), line);
    fo.line = line;
    out.forces.push_back(fo);
  }
  // PARAM: output options only on this path
}

// Cards whose first line lies in [l0, l1) of lines[.. end).
void parse_chunk(Bdf::Chunk& out, const std::vector<sv>& lines, size_t l0, size_t l1,
                 size_t end) {
  std::vector<sv> f;
  f.reserve(64);
  try {
    for (size_t i = l0; i < l1; ++i) {
      const sv l = lines[i];
      if (is_comment_line(l) || is_continuation(l)) continue;
      f.clear();
      split_line(l, f);
      const long long line = static_cast<long long>(i) + 1;
      size_t j = i + 1;
      for (; j < end; ++j) {
        const sv nx = lines[j];
        if (is_comment_line(nx)) continue;
        if (!is_continuation(nx)) break;
        const size_t c0 = f.size();
        split_line(nx, f);
        // drop the continuation's marker field, keep its fields 1-8
        const size_t got = f.size() - c0;
        if (got > 9) f.resize(c0 + 9);
        f.erase(f.begin() + static_cast<long>(c0));
      }
      i = j - 1;
      ++out.cards;
      if (f.empty()) continue;
      const std::string kw = card_keyword(f[0]);
      if (kw.empty()) continue;
      switch (classify(kw)) {
        case Kind::Path:
          process_card(out, kw, f, line);
          break;
        case Kind::Element:
          out.outside.push_back({kw, -1, line});
          break;
        case Kind::SetCard: {
          int sid = -1;
          if (f.size() > 1 && !f[1].empty()) {
            try {
              sid = parse_int(f[1], line);
            } catch (const ParseFail&) {
              sid = -1;
            }
          }
          out.outside.push_back({kw, sid, line});
          break;
        }
        case Kind::Harmless:
          break;
        case Kind::Ignored:
          out.ignored.insert(kw);
          break;
      }
    }
  } catch (const ParseFail& e) {
    out.failed = true;
    out.fail = e;
  }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
      .count();
}

void parse_bulk(Bdf& d, const std::vector<sv>& lines, size_t b, size_t e, int threads) {
  const size_t n = e > b ? e - b : 0;
  int T = thread_count(threads);
  if (n < 20000) T = 1;
  if (static_cast<size_t>(T) > n / 4096 + 1) T = static_cast<int>(n / 4096 + 1);
  d.threads = T;
  // chunk starts moved forward to card starts
  std::vector<size_t> st(static_cast<size_t>(T) + 1, e);
  st[0] = b;
  for (int k = 1; k < T; ++k) {
    size_t s = b + n * static_cast<size_t>(k) / static_cast<size_t>(T);
    s = std::max(s, st[static_cast<size_t>(k) - 1]);
    while (s < e && (is_comment_line(lines[s]) || is_continuation(lines[s]))) ++s;
    st[static_cast<size_t>(k)] = s;
  }
  std::vector<Bdf::Chunk> ch(static_cast<size_t>(T));
  if (T == 1) {
    parse_chunk(ch[0], lines, b, e, e);
  } else {
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(T));
    for (int k = 0; k < T; ++k)
      pool.emplace_back(parse_chunk, std::ref(ch[static_cast<size_t>(k)]), std::cref(lines),
                        st[static_cast<size_t>(k)], st[static_cast<size_t>(k) + 1], e);
    for (auto& t : pool) t.join();
  }
  // the first failure in file order
  const Bdf::Chunk* bad = nullptr;
  for (const auto& c : ch)
    if (c.failed && (!bad || c.fail.line < bad->fail.line)) bad = &c;
  if (bad) throw bad->fail;
  auto cat = [](auto& dst, auto& src) { dst.insert(dst.end(), src.begin(), src.end()); };
  size_t ng = 0, nh = 0;
  for (const auto& c : ch) {
    ng += c.grids.size();
    nh += c.hexas.size();
  }
  d.all.grids.reserve(ng);
  d.all.hexas.reserve(nh);
  for (auto& c : ch) {
    cat(d.all.grids, c.grids);
    cat(d.all.hexas, c.hexas);
    cat(d.all.mats, c.mats);
    cat(d.all.props, c.props);
    cat(d.all.spcs, c.spcs);
    cat(d.all.forces, c.forces);
    cat(d.all.outside, c.outside);
    d.all.ignored.insert(c.ignored.begin(), c.ignored.end());
    d.cards += c.cards;
  }
}

std::string line_tag(long long line) { return "line " + std::to_string(line); }

// id -> position of the last record with that id: a table when the ids are
// dense, else a hash map.
struct IdIndex {
  bool dense = false;
  int lo = 0;
  std::vector<int> table;
  std::unordered_map<int, int> hmap;
  template <typename R, typename Key>
  void build(const std::vector<R>& recs, Key key) {
    if (recs.empty()) return;
    long long mn = LLONG_MAX, mx = LLONG_MIN;
    for (const auto& r : recs) {
      mn = std::min<long long>(mn, key(r));
      mx = std::max<long long>(mx, key(r));
    }
    dense = mx - mn < 8LL * static_cast<long long>(recs.size()) + 4096;
    if (dense) {
      lo = static_cast<int>(mn);
      table.assign(static_cast<size_t>(mx - mn) + 1, -1);
      for (size_t i = 0; i < recs.size(); ++i)
        table[static_cast<size_t>(key(recs[i]) - lo)] = static_cast<int>(i);
    } else {
      hmap.reserve(recs.size() * 2);
      for (size_t i = 0; i < recs.size(); ++i) hmap[key(recs[i])] = static_cast<int>(i);
    }
  }
  int find(int id) const {
    if (dense) {
      const long long k = static_cast<long long>(id) - lo;
      return (k >= 0 && k < static_cast<long long>(table.size())) ? table[static_cast<size_t>(k)]
                                                                   : -1;
    }
    const auto it = hmap.find(id);
    return it == hmap.end() ? -1 : it->second;
  }
};

// Mesh arrays of the deck; model_error says why they cannot be formed.
void form_mesh(Bdf& d) {
  auto fail = [&](std::string m) {
    if (d.model_error.empty()) d.model_error = std::move(m);
  };
  if (d.sol == 103) fail("SOL 103 (modes) is outside the SOL 101 path");
  for (const auto& o : d.all.outside)
    if (o.sid < 0) {
      fail("card " + o.kw + " (" + line_tag(o.line) +
           ") is outside the CHEXA8 SOL 101 path (CHEXA8 elements only)");
      break;
    }
  // nodes sorted by id; a repeated id keeps its last card (map insertion)
  const auto& G = d.all.grids;
  // record positions in ascending id order, one per id (its last card):
  // through an id table when the ids are dense, else a sort
  std::vector<int> pick;
  {
    IdIndex gi;
    gi.build(G, [](const Bdf::Grid& g) { return g.id; });
    pick.reserve(G.size());
    if (gi.dense) {
      for (int p : gi.table)
        if (p >= 0) pick.push_back(p);
    } else {
      std::vector<std::pair<int, int>> order(G.size());
      for (size_t i = 0; i < G.size(); ++i) order[i] = {G[i].id, static_cast<int>(i)};
      std::sort(order.begin(), order.end());
      for (size_t i = 0; i < order.size(); ++i)
        if (i + 1 == order.size() || order[i + 1].first != order[i].first)
          pick.push_back(order[i].second);
    }
  }
  d.node_ids.clear();
  d.xyz.clear();
  d.node_ids.reserve(pick.size());
  d.xyz.reserve(3 * pick.size());
  for (const int pi : pick) {
    const auto& g = G[static_cast<size_t>(pi)];
    if (g.cp != 0 || g.cd != 0)
      fail("GRID " + std::to_string(g.id) + " (" + line_tag(g.line) +
           "): coordinate systems (CP / CD) are outside this path");
    d.node_ids.push_back(g.id);
    d.xyz.insert(d.xyz.end(), g.x, g.x + 3);
  }
  const size_t N = d.node_ids.size();
  // id -> index: a table when the ids are dense, else a hash map
  const long long max_id = N ? d.node_ids.back() : 0;
  const long long min_id = N ? d.node_ids.front() : 0;
  std::vector<int> table;
  std::unordered_map<int, int> hmap;
  const bool dense = N && min_id >= 0 && max_id < 8LL * static_cast<long long>(N) + 4096;
  if (dense) {
    table.assign(static_cast<size_t>(max_id) + 1, -1);
    for (size_t i = 0; i < N; ++i) table[static_cast<size_t>(d.node_ids[i])] = static_cast<int>(i);
  } else {
    hmap.reserve(N * 2);
    for (size_t i = 0; i < N; ++i) hmap[d.node_ids[i]] = static_cast<int>(i);
  }
  auto node_index = [&](int id) -> int {
    if (dense) return (id >= 0 && id <= max_id) ? table[static_cast<size_t>(id)] : -1;
    const auto it = hmap.find(id);
    return it == hmap.end() ? -1 : it->second;
  };
  // MID -> MAT1 and PID -> PSOLID, the last card of an id winning
  IdIndex mats, props;
  mats.build(d.all.mats, [](const Bdf::Mat1& m) { return m.mid; });
  props.build(d.all.props, [](const Bdf::Psolid& p) { return p.pid; });
  const auto& H = d.all.hexas;
  d.elem_ids.resize(H.size());
  d.conn.resize(8 * H.size());
  d.E.resize(H.size());
  d.nu.resize(H.size());
  d.form.resize(H.size());
  int last_pid = INT_MIN, last_isop = VSGB_EAS;
  double last_E = 0.0, last_nu = 0.0;
  for (size_t e = 0; e < H.size() && d.model_error.empty(); ++e) {
    const auto& h = H[e];
    d.elem_ids[e] = h.eid;
    for (int k = 0; k < 8; ++k) {
      const int idx = node_index(h.g[k]);
      if (idx < 0) {
        fail("CHEXA " + std::to_string(h.eid) + " (" + line_tag(h.line) + "): GRID " +
             std::to_string(h.g[k]) + " is not defined");
        break;
      }
      d.conn[8 * e + static_cast<size_t>(k)] = idx;
    }
    if (h.pid != last_pid) {
      const int pi = props.find(h.pid);
      if (pi < 0) {
        fail("CHEXA " + std::to_string(h.eid) + " (" + line_tag(h.line) + "): PSOLID " +
             std::to_string(h.pid) + " is not defined");
        break;
      }
      const auto& pr = d.all.props[static_cast<size_t>(pi)];
      const int mi = mats.find(pr.mid);
      if (mi < 0) {
        fail("PSOLID " + std::to_string(h.pid) + ": MAT1 " + std::to_string(pr.mid) +
             " is not defined");
        break;
      }
      last_pid = h.pid;
      last_isop = pr.isop;
      last_E = d.all.mats[static_cast<size_t>(mi)].E;
      last_nu = d.all.mats[static_cast<size_t>(mi)].nu;
    }
    d.E[e] = last_E;
    d.nu[e] = last_nu;
    d.form[e] = last_isop;
  }
  std::string w;
  auto join = [](const std::set<std::string>& s) {
    std::string o;
    for (const auto& k : s) o += (o.empty() ? "" : ", ") + k;
    return o;
  };
  if (!d.ignored_case.empty()) w += "Case control: " + join(d.ignored_case);
  if (!d.all.ignored.empty()) w += std::string(w.empty() ? "" : "\n") + "Bulk data: " + join(d.all.ignored);
  if (!w.empty()) w = "Unsupported BDF cards were ignored (unique keywords only):\n" + w;
  d.warnings = w;
}

void read_deck(Bdf& d, sv text, int threads) {
  const auto t0 = std::chrono::steady_clock::now();
  const std::vector<sv> lines = split_lines(text, thread_count(threads));
  d.lines = static_cast<long long>(lines.size());
  size_t b = 0, e = 0;
  find_markers(d, lines, &b, &e);
  parse_case_control(d, lines, b);
  d.lines_ms = ms_since(t0);
  const auto t1 = std::chrono::steady_clock::now();
  parse_bulk(d, lines, b, e, threads);
  d.cards_ms = ms_since(t1);
  const auto t2 = std::chrono::steady_clock::now();
  form_mesh(d);
  d.mesh_ms = ms_since(t2);
  d.parse_ms = ms_since(t0);
}

void copy_msg(const std::string& m, char* buf, size_t len) {
  if (!buf || len == 0) return;
  const size_t n = std::min(m.size(), len - 1);
  std::memcpy(buf, m.data(), n);
  buf[n] = '\0';
}

int make(sv text, int threads, vsgb_bdf** out, char* err, size_t err_len, double read_ms) {
  auto* d = new (std::nothrow) vsgb_bdf();
  if (!d) return VSGB_ERR_LIMIT;
  try {
    d->read_ms = read_ms;
    read_deck(*d, text, threads);
  } catch (const ParseFail& f) {
    copy_msg(f.line > 0 ? "Line " + std::to_string(f.line) + ": " + f.msg : f.msg, err, err_len);
    delete d;
    return VSGB_ERR_INVALID;
  } catch (const std::bad_alloc&) {
    copy_msg("out of host memory while reading the deck", err, err_len);
    delete d;
    return VSGB_ERR_LIMIT;
  } catch (const std::exception& x) {
    copy_msg(x.what(), err, err_len);
    delete d;
    return VSGB_ERR_INVALID;
  }
  *out = d;
  return VSGB_OK;
}

// Checks of subcase s for its constraint / load sets; "" when usable.
std::string subcase_problem(const Bdf& d, int s) {
  if (s < 0 || s >= static_cast<int>(d.subcases.size())) return "subcase index out of range";
  const auto& sc = d.subcases[static_cast<size_t>(s)];
  const std::string id = "subcase " + std::to_string(sc.id);
  if (sc.mpc != 0) return id + ": MPC set " + std::to_string(sc.mpc) + " is outside this path";
  const int temp_set = sc.temp != 0 ? sc.temp : sc.load;
  for (const auto& o : d.all.outside) {
    if (o.sid < 0) continue;
    const bool spc = o.kw == "SPC", temp = o.kw == "TEMP" || o.kw == "TEMPD";
    const int set = spc ? sc.spc : temp ? temp_set : sc.load;
    if (o.sid == set)
      return id + ": " + o.kw + " (" + line_tag(o.line) + ") of its " +
             (spc ? "SPC" : temp ? "temperature" : "LOAD") + " set (thermal and other "
             "loads than FORCE are outside this path)";
  }
  for (const auto& f : d.all.forces)
    if (f.sid == sc.load && f.cid != 0)
      return id + ": FORCE (" + line_tag(f.line) + ") in coordinate system " +
             std::to_string(f.cid) + " is outside this path";
  return "";
}

}  // namespace

// ── C ABI ─────────────────────────────────────────────────────────────────

extern "C" {

int vsgb_bdf_read(const char* path, int threads, vsgb_bdf** out, char* err, size_t err_len) {
  if (!path || !out) {
    copy_msg("vsgb_bdf_read: invalid argument", err, err_len);
    return VSGB_ERR_INVALID;
  }
  *out = nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  std::FILE* fp = std::fopen(path, "rb");
  if (!fp) {
    copy_msg(std::string("Cannot open BDF file: ") + path, err, err_len);
    return VSGB_ERR_INVALID;
  }
  std::string text;
  long sz = -1;
  if (std::fseek(fp, 0, SEEK_END) == 0) {
    sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
  }
  if (sz > 0) {
    text.resize(static_cast<size_t>(sz));
    text.resize(std::fread(text.data(), 1, text.size(), fp));
  }
  char buf[1 << 16];
  for (;;) {  // whatever follows (or a stream without a size)
    const size_t got = std::fread(buf, 1, sizeof(buf), fp);
    if (got == 0) break;
    text.append(buf, got);
  }
  const bool bad = std::ferror(fp) != 0;
  std::fclose(fp);
  if (bad) {
    copy_msg(std::string("Cannot read BDF file: ") + path, err, err_len);
    return VSGB_ERR_INVALID;
  }
  return make(text, threads, out, err, err_len, ms_since(t0));
}

int vsgb_bdf_parse(const char* text, size_t len, int threads, vsgb_bdf** out, char* err,
                   size_t err_len) {
  if ((!text && len) || !out) {
    copy_msg("vsgb_bdf_parse: invalid argument", err, err_len);
    return VSGB_ERR_INVALID;
  }
  *out = nullptr;
  return make(sv(text ? text : "", len), threads, out, err, err_len, 0.0);
}

void vsgb_bdf_free(vsgb_bdf* d) { delete d; }

int vsgb_bdf_info(vsgb_bdf* d, vsgb_bdf_stats* info) {
  if (!d || !info) return VSGB_ERR_INVALID;
  info->n_nodes = static_cast<int>(d->node_ids.size());
  info->n_elem = static_cast<int>(d->all.hexas.size());
  info->n_subcases = static_cast<int>(d->subcases.size());
  info->sol = d->sol;
  info->lines = d->lines;
  info->cards = d->cards;
  info->threads = d->threads;
  info->read_ms = d->read_ms;
  info->parse_ms = d->parse_ms;
  info->mesh_ok = d->model_error.empty() ? 1 : 0;
  info->lines_ms = d->lines_ms;
  info->cards_ms = d->cards_ms;
  info->mesh_ms = d->mesh_ms;
  return VSGB_OK;
}

int vsgb_bdf_message(vsgb_bdf* d, int which, char* buf, size_t len) {
  if (!d || !buf || len == 0) return VSGB_ERR_INVALID;
  copy_msg(which == 0 ? d->model_error : which == 1 ? d->warnings : d->last_error, buf, len);
  return VSGB_OK;
}

int vsgb_bdf_subcase(vsgb_bdf* d, int s, int* id, int* load_set, int* spc_set) {
  if (!d || s < 0 || s >= static_cast<int>(d->subcases.size())) return VSGB_ERR_INVALID;
  const auto& sc = d->subcases[static_cast<size_t>(s)];
  if (id) *id = sc.id;
  if (load_set) *load_set = sc.load;
  if (spc_set) *spc_set = sc.spc;
  return VSGB_OK;
}

int vsgb_bdf_mesh(vsgb_bdf* d, int* node_ids, double* xyz, int* elem_ids, int* conn, double* E,
                  double* nu, int* form) {
  if (!d) return VSGB_ERR_INVALID;
  if (!d->model_error.empty()) {
    d->last_error = d->model_error;
    return VSGB_ERR_INVALID;
  }
  const size_t N = d->node_ids.size(), M = d->all.hexas.size();
  if (node_ids) std::memcpy(node_ids, d->node_ids.data(), sizeof(int) * N);
  if (xyz) std::memcpy(xyz, d->xyz.data(), sizeof(double) * 3 * N);
  if (elem_ids) std::memcpy(elem_ids, d->elem_ids.data(), sizeof(int) * M);
  if (conn) std::memcpy(conn, d->conn.data(), sizeof(int) * 8 * M);
  if (E) std::memcpy(E, d->E.data(), sizeof(double) * M);
  if (nu) std::memcpy(nu, d->nu.data(), sizeof(double) * M);
  if (form) std::memcpy(form, d->form.data(), sizeof(int) * M);
  return VSGB_OK;
}

int vsgb_bdf_constraints(vsgb_bdf* d, int s, int* count, int* nodes, int* masks) {
  if (!d || !count) return VSGB_ERR_INVALID;
  const std::string why = subcase_problem(*d, s);
  if (!why.empty()) {
    d->last_error = why;
    return VSGB_ERR_INVALID;
  }
  const int sid = d->subcases[static_cast<size_t>(s)].spc;
  int k = 0;
  for (const auto& c : d->all.spcs) {
    if (c.sid != sid) continue;
    if (nodes) nodes[k] = c.node;
    if (masks) masks[k] = c.mask;
    ++k;
  }
  *count = k;
  return VSGB_OK;
}

int vsgb_bdf_forces(vsgb_bdf* d, int s, int* count, int* nodes, double* scale, double* dir) {
  if (!d || !count) return VSGB_ERR_INVALID;
  const std::string why = subcase_problem(*d, s);
  if (!why.empty()) {
    d->last_error = why;
    return VSGB_ERR_INVALID;
  }
  const int sid = d->subcases[static_cast<size_t>(s)].load;
  int k = 0;
  for (const auto& f : d->all.forces) {
    if (f.sid != sid) continue;
    if (nodes) nodes[k] = f.node;
    if (scale) scale[k] = f.scale;
    if (dir)
      for (int c = 0; c < 3; ++c) dir[3 * k + c] = f.dir[c];
    ++k;
  }
  *count = k;
  return VSGB_OK;
}

}  // extern "C"
