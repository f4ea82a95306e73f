// sg_sasl.cpp -- SASL shader source to a C++ shader body.
//
// The reference compiles SASL (its HLSL-like shader language) with an LLVM
// JIT into the shader units its CPU pipeline calls (renderer.cpp:41-58
// compile(); sasl/src/{parser,semantic,codegen}; shader_unit.cpp:28-186).
// Here a SASL vertex or pixel shader becomes the C++ class the GPU pipeline
// takes as a user shader module (salvia_gb300/device_shader.cuh), written
// against salvia_gb300/sasl_rt.cuh, and built like any other module: nvcc
// for the pass kernels and the host body, or a host compiler for the body
// alone.  One pass over the tokens emits the class; what the source cannot
// mean in that form is refused with a line-numbered message.
//
// The language accepted: struct declarations with member semantics
// (TEXCOORD(0), TEXCOORD0, COLOR, SV_Position, SV_Target ...); global
// uniforms (scalars, vectors, matrices) and samplers; static const globals;
// functions with in / out / inout parameters and semantics; local
// declarations with initialisers and initialiser lists; if / else, for,
// while, do-while, switch, break, continue, return; the C operators with
// their precedence, casts, constructors (float4(a, b)), swizzles and write
// masks, indexing; the intrinsics of sasl_rt.cuh and ddx / ddy, tex2D,
// tex2Dgrad, tex2Dlod.
//
// The stage interface (reported in the reflection text, one item a line):
//  - vertex inputs take input registers 0, 1, ... in the order their
//    semantics appear in the entry's parameters; the output with semantic
//    SV_Position / POSITION is the position and the other outputs take
//    varying registers 0, 1, ... in order (at most SG_MAX_VARYINGS);
//  - pixel inputs are linked to varyings by constant word 47: three bits per
//    input in order of appearance holding 1 + the register, 0 meaning the
//    input's own order (link() in salviarenderer_gb300/sasl.py fills it
//    from a vertex shader's reflection); SV_Position reads the position;
//    outputs COLOR(n) / SV_Target(n) write colour target n;
//  - uniforms take consecutive 32-bit constant words in declaration order
//    (a matrix row by row), 47 words at most in a pixel shader, 48 in a
//    vertex shader, loaded into the invocation's own copies at entry (a
//    shader may assign to them); a stage samples through sampler slot 0, so
//    it may use one sampler.
// ddx / ddy (and tex2D, which takes the derivatives of its coordinate,
// cg_impl.cpp:902-908) apply to a pixel-shader input read directly in the
// entry function (in.uv, in.uv.xy): the pipeline gives the quad's
// differences of an interpolated register (cpp_pixel_shader.cpp:13-19), not
// of computed values.  tex2Dbias, tex2Dproj and texCUBE* are refused: the
// reference's pixel-shader bindings for them are unimplemented
// (sampler_api.cpp:21-70).
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "salvia_gb300.h"

namespace {

struct SaslError {
  int line;
  std::string msg;
};

struct Token {
  enum Kind { End, Id, Int, Float, Punct } kind;
  std::string text;
  int line;
};

std::vector<Token> lex(std::string const& s) {
  static char const* const multi[] = {"<<=", ">>=", "++", "--", "+=", "-=", "*=", "/=", "%=", "&=", "|=",
                                      "^=",  "<<",  ">>", "<=", ">=", "==", "!=", "&&", "||"};
  std::vector<Token> out;
  int line = 1;
  size_t i = 0, n = s.size();
  while (i < n) {
    char c = s[i];
    if (c == '\n') {
      ++line;
      ++i;
    } else if (std::isspace(static_cast<unsigned char>(c))) {
      ++i;
    } else if (c == '/' && i + 1 < n && s[i + 1] == '/') {
      while (i < n && s[i] != '\n') ++i;
    } else if (c == '/' && i + 1 < n && s[i + 1] == '*') {
      i += 2;
      while (i + 1 < n && !(s[i] == '*' && s[i + 1] == '/')) {
        if (s[i] == '\n') ++line;
        ++i;
      }
      if (i + 1 >= n) throw SaslError{line, "unterminated comment"};
      i += 2;
    } else if (c == '#') {
      throw SaslError{line, "preprocessor directives are not supported"};
    } else if (std::isalpha(static_cast<unsigned char>(c)) || c == '_') {
      size_t j = i;
      while (j < n && (std::isalnum(static_cast<unsigned char>(s[j])) || s[j] == '_')) ++j;
      out.push_back({Token::Id, s.substr(i, j - i), line});
      i = j;
    } else if (std::isdigit(static_cast<unsigned char>(c)) ||
               (c == '.' && i + 1 < n && std::isdigit(static_cast<unsigned char>(s[i + 1])))) {
      size_t j = i;
      bool fl = false;
      if (c == '0' && j + 1 < n && (s[j + 1] == 'x' || s[j + 1] == 'X')) {
        j += 2;
        while (j < n && std::isxdigit(static_cast<unsigned char>(s[j]))) ++j;
      } else {
        while (j < n && std::isdigit(static_cast<unsigned char>(s[j]))) ++j;
        if (j < n && s[j] == '.') {
          fl = true;
          ++j;
          while (j < n && std::isdigit(static_cast<unsigned char>(s[j]))) ++j;
        }
        if (j < n && (s[j] == 'e' || s[j] == 'E')) {
          size_t k = j + 1;
          if (k < n && (s[k] == '+' || s[k] == '-')) ++k;
          if (k < n && std::isdigit(static_cast<unsigned char>(s[k]))) {
            fl = true;
            j = k;
            while (j < n && std::isdigit(static_cast<unsigned char>(s[j]))) ++j;
          }
        }
      }
      std::string num = s.substr(i, j - i), suffix;
      while (j < n && std::isalpha(static_cast<unsigned char>(s[j]))) suffix += s[j++];
      for (char& ch : suffix) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
      if (suffix == "f" || suffix == "h") {
        fl = true;
      } else if (suffix == "u" || suffix == "ul" || suffix == "lu") {
        num += "u";
      } else if (!suffix.empty() && suffix != "l") {
        throw SaslError{line, "bad numeric literal suffix '" + suffix + "'"};
      }
      if (fl) {
        if (num.back() == '.') num += "0";
        if (num[0] == '.') num = "0" + num;
        num += "f";
      }
      out.push_back({fl ? Token::Float : Token::Int, num, line});
      i = j;
    } else {
      bool matched = false;
      for (char const* m : multi) {
        size_t len = std::strlen(m);
        if (s.compare(i, len, m) == 0) {
          out.push_back({Token::Punct, m, line});
          i += len;
          matched = true;
          break;
        }
      }
      if (!matched) {
        if (!std::strchr("{}()[];,.:?=+-*/%<>!~&|^", c)) throw SaslError{line, std::string("unexpected character '") + c + "'"};
        out.push_back({Token::Punct, std::string(1, c), line});
        ++i;
      }
    }
  }
  out.push_back({Token::End, "", line});
  return out;
}

struct Type {
  enum Kind { Unknown, Void, Scalar, Vector, Matrix, Struct, Sampler } kind = Unknown;
  std::string base;  // float, double, int, uint, bool
  int rows = 1, cols = 1;
  std::string sname;
  int array = 0;
  int comps() const { return kind == Scalar ? 1 : kind == Vector ? cols : kind == Matrix ? rows * cols : 0; }
  std::string elem_cpp() const {
    if (base == "float") return "float";
    if (base == "double") return "double";
    if (base == "int") return "int32_t";
    if (base == "uint") return "uint32_t";
    return "bool";
  }
  std::string cpp() const {
    switch (kind) {
      case Void: return "void";
      case Scalar: return elem_cpp();
      case Vector: return "sasl_rt::vec<" + elem_cpp() + ", " + std::to_string(cols) + ">";
      case Matrix:
        return "sasl_rt::mat<" + elem_cpp() + ", " + std::to_string(rows) + ", " + std::to_string(cols) + ">";
      case Struct: return "S_" + sname;
      default: return "void";
    }
  }
  bool numeric() const { return kind == Scalar || kind == Vector || kind == Matrix; }
};

Type type_from_name(std::string const& t) {
  Type ty;
  if (t == "void") {
    ty.kind = Type::Void;
    return ty;
  }
  if (t == "sampler" || t == "sampler1D" || t == "sampler2D" || t == "sampler3D" || t == "samplerCUBE") {
    ty.kind = Type::Sampler;
    return ty;
  }
  static char const* const bases[] = {"bool", "int", "uint", "half", "float", "double"};
  for (char const* b : bases) {
    size_t const bl = std::strlen(b);
    if (t.compare(0, bl, b) != 0) continue;
    std::string rest = t.substr(bl);
    ty.base = std::string(b) == "half" ? "float" : b;
    if (rest.empty()) {
      ty.kind = Type::Scalar;
      return ty;
    }
    if (rest.size() == 1 && rest[0] >= '1' && rest[0] <= '4') {
      ty.kind = Type::Vector;
      ty.cols = rest[0] - '0';
      return ty;
    }
    if (rest.size() == 3 && rest[0] >= '1' && rest[0] <= '4' && rest[1] == 'x' && rest[2] >= '1' && rest[2] <= '4') {
      ty.kind = Type::Matrix;
      ty.rows = rest[0] - '0';
      ty.cols = rest[2] - '0';
      return ty;
    }
  }
  return ty;
}

struct Semantic {
  bool present = false;
  std::string name;  // upper case, without the index
  int index = 0;
};

struct Member {
  std::string name;
  Type type;
  Semantic sem;
};

struct Param {
  std::string name;
  Type type;
  Semantic sem;
  bool out = false, in = true;
};

struct Func {
  std::string name;
  Type ret;
  Semantic ret_sem;
  std::vector<Param> params;
};

// what an expression is, besides its code
struct Expr {
  std::string code;
  Type type;
  bool lvalue = false;
  bool sampler = false;
  std::string sampler_name;
  // a write mask of several components: its base and indices
  bool multi = false;
  std::string multi_base, multi_idx;
  // a pixel-shader input read directly: its link slot, declared type and
  // the swizzles applied since
  int vary = -1;
  Type vary_type;
  std::vector<std::string> vary_wrap;
  // an entry-function struct parameter holding pixel inputs
  std::map<std::string, int> const* members_vary = nullptr;
  std::map<std::string, Type> const* members_type = nullptr;
};

struct Sym {
  enum Kind { Local, Uniform, Sampler, Const } kind = Local;
  Type type;
  std::string code;
  int vary = -1;  // a scalar pixel input parameter of the entry
  std::map<std::string, int> members_vary;
  std::map<std::string, Type> members_type;
};

struct IoItem {
  Semantic sem;
  Type type;
  std::string path;
};

std::string upper(std::string s) {
  for (char& c : s) c = static_cast<char>(std::toupper(static_cast<unsigned char>(c)));
  return s;
}

class Translator {
 public:
  Translator(std::string const& src, int lang, std::string entry, std::string cls)
      : toks_(lex(src)), lang_(lang), entry_(std::move(entry)), cls_(std::move(cls)) {}

  void run(std::string& source, std::string& reflection) {
    if (lang_ != SG_LANG_VERTEX_SHADER && lang_ != SG_LANG_PIXEL_SHADER)
      throw SaslError{0, "only vertex and pixel shaders translate to shader modules"};
    pick_entry();
    scopes_.emplace_back();
    while (peek().kind != Token::End) top_level();
    if (!have_entry_) throw SaslError{0, "entry function '" + entry_ + "' not found"};
    emit(source, reflection);
  }

 private:
  std::vector<Token> toks_;
  size_t pos_ = 0;
  int lang_;
  std::string entry_, cls_;
  std::map<std::string, std::vector<Member>> structs_;
  std::vector<std::string> struct_order_;
  std::map<std::string, std::vector<Func>> funcs_;
  std::vector<std::map<std::string, Sym>> scopes_;
  std::ostringstream structs_out_, members_out_, refl_, uniform_loads_;
  int next_word_ = 0;
  std::set<std::string> samplers_used_;
  bool in_entry_ = false, have_entry_ = false;
  Func entry_func_;
  Type cur_ret_;
  int npsin_ = 0;  // pixel inputs linked so far

  bool vs() const { return lang_ == SG_LANG_VERTEX_SHADER; }

  Token const& peek(size_t k = 0) const { return toks_[std::min(pos_ + k, toks_.size() - 1)]; }
  Token const& next() {
    Token const& t = toks_[pos_];
    if (pos_ + 1 < toks_.size()) ++pos_;
    return t;
  }
  [[noreturn]] void fail(std::string const& msg) const { throw SaslError{peek().line, msg}; }
  bool is(char const* p) const { return peek().kind != Token::End && peek().text == p && peek().kind != Token::Float && peek().kind != Token::Int; }
  bool accept(char const* p) {
    if (is(p)) {
      next();
      return true;
    }
    return false;
  }
  void expect(char const* p) {
    if (!accept(p)) fail(std::string("expected '") + p + "' before '" + peek().text + "'");
  }
  std::string expect_id() {
    if (peek().kind != Token::Id) fail("expected a name before '" + peek().text + "'");
    return next().text;
  }

  // the entry: the named function, else main / vs_main / ps_main, else the
  // last function defined
  void pick_entry() {
    std::vector<std::string> names;
    int depth = 0;
    for (size_t i = 0; i + 1 < toks_.size(); ++i) {
      Token const& t = toks_[i];
      if (t.kind == Token::Punct && (t.text == "{" || t.text == "(")) ++depth;
      if (t.kind == Token::Punct && (t.text == "}" || t.text == ")")) --depth;
      if (depth == 0 && i > 0 && t.kind == Token::Id && toks_[i + 1].text == "(" && toks_[i - 1].kind == Token::Id)
        names.push_back(t.text);
    }
    if (!entry_.empty()) return;
    for (char const* pref : {"main", vs() ? "vs_main" : "ps_main"})
      for (auto const& n : names)
        if (n == pref) {
          entry_ = n;
          return;
        }
    if (names.empty()) throw SaslError{0, "no function to be the entry"};
    entry_ = names.back();
  }

  Sym const* lookup(std::string const& n) const {
    for (auto it = scopes_.rbegin(); it != scopes_.rend(); ++it) {
      auto f = it->find(n);
      if (f != it->end()) return &f->second;
    }
    return nullptr;
  }

  bool is_type_start() const {
    if (peek().kind != Token::Id) return false;
    std::string const& t = peek().text;
    if (t == "const" || t == "static" || t == "uniform" || t == "struct") return true;
    if (structs_.count(t)) return true;
    return type_from_name(t).kind != Type::Unknown;
  }

  Type parse_type() {
    accept("struct");
    std::string const t = expect_id();
    if (structs_.count(t)) {
      Type ty;
      ty.kind = Type::Struct;
      ty.sname = t;
      return ty;
    }
    Type ty = type_from_name(t);
    if (ty.kind == Type::Unknown) fail("unknown type '" + t + "'");
    return ty;
  }

  Semantic parse_semantic() {
    Semantic s;
    s.present = true;
    std::string n = upper(expect_id());
    size_t d = n.size();
    while (d > 0 && std::isdigit(static_cast<unsigned char>(n[d - 1]))) --d;
    if (d < n.size()) {
      s.index = std::atoi(n.c_str() + d);
      n = n.substr(0, d);
    }
    if (accept("(")) {
      if (peek().kind != Token::Int) fail("expected a semantic index");
      s.index = std::atoi(next().text.c_str());
      expect(")");
    }
    s.name = n;
    return s;
  }

  int parse_array_len() {
    if (!accept("[")) return 0;
    if (peek().kind != Token::Int) fail("array lengths must be integer literals");
    int const n = std::atoi(next().text.c_str());
    if (n <= 0 || n > 4096) fail("bad array length");
    expect("]");
    return n;
  }

  // ---- top level -------------------------------------------------------------
  void top_level() {
    if (accept(";")) return;
    if (is("struct") && peek(2).text == "{") {
      parse_struct();
      return;
    }
    bool is_static = false, is_const = false;
    for (;;) {
      if (accept("uniform") || accept("extern")) continue;
      if (accept("static")) {
        is_static = true;
        continue;
      }
      if (accept("const")) {
        is_const = true;
        continue;
      }
      break;
    }
    Type ty = parse_type();
    std::string const name = expect_id();
    if (is("(")) {
      parse_function(ty, name);
      return;
    }
    for (std::string n = name;;) {
      global_decl(ty, n, is_static || is_const);
      if (!accept(",")) break;
      n = expect_id();
    }
    expect(";");
  }

  void parse_struct() {
    expect("struct");
    std::string const name = expect_id();
    if (structs_.count(name)) fail("struct '" + name + "' redefined");
    expect("{");
    std::vector<Member> ms;
    structs_out_ << "struct S_" << name << " {\n";
    while (!accept("}")) {
      Type ty = parse_type();
      if (ty.kind == Type::Sampler || ty.kind == Type::Void) fail("bad struct member type");
      for (;;) {
        Member m;
        m.name = expect_id();
        m.type = ty;
        m.type.array = parse_array_len();
        if (accept(":")) m.sem = parse_semantic();
        structs_out_ << "  " << m.type.cpp() << " m_" << m.name << (m.type.array ? "[" + std::to_string(m.type.array) + "]" : "")
                     << "{};\n";
        ms.push_back(m);
        if (!accept(",")) break;
      }
      expect(";");
    }
    accept(";");
    structs_out_ << "};\n";
    structs_[name] = ms;
    struct_order_.push_back(name);
  }

  void global_decl(Type ty, std::string const& name, bool constant) {
    ty.array = parse_array_len();
    if (accept(":")) parse_semantic();  // register bindings are ignored
    Sym s;
    s.type = ty;
    if (ty.kind == Type::Sampler) {
      if (ty.array) fail("sampler arrays are not supported");
      s.kind = Sym::Sampler;
      refl_ << "sampler " << name << " 0\n";
    } else if (constant) {
      if (!accept("=")) fail("a static or const global needs an initialiser");
      if (ty.array || !ty.numeric()) fail("static const globals must be scalars, vectors or matrices");
      Expr e = parse_assign();
      s.kind = Sym::Const;
      s.code = "k_" + name + "()";
      members_out_ << "  __host__ __device__ " << ty.cpp() << " k_" << name << "() const { return sasl_rt::cast<"
                   << ty.cpp() << ">(" << e.code << "); }\n";
    } else {
      if (ty.array || !ty.numeric()) fail("uniform '" + name + "': uniforms must be scalars, vectors or matrices");
      if (is("=")) fail("uniform '" + name + "' cannot have an initialiser");
      int const words = ty.comps();
      int const cap = vs() ? SG_MAX_SHADER_CONSTANTS : SG_MAX_SHADER_CONSTANTS - 1;
      if (next_word_ + words > cap) fail("uniforms exceed the stage's " + std::to_string(cap) + " constant words");
      // an invocation's own copy, loaded at entry: a shader may assign to it
      s.kind = Sym::Uniform;
      s.code = "u_" + name;
      std::string const e = ty.elem_cpp();
      members_out_ << "  mutable " << ty.cpp() << " u_" << name << ";\n";
      if (ty.kind == Type::Scalar) {
        uniform_loads_ << "    u_" << name << " = sasl_rt::from_word<" << e << ">(constant(" << next_word_ << "));\n";
      } else {
        uniform_loads_ << "    for (int i = 0; i < " << words << "; ++i) u_" << name
                       << (ty.kind == Type::Vector ? ".v[i]" : ".r[i / " + std::to_string(ty.cols) + "].v[i % " + std::to_string(ty.cols) + "]")
                       << " = sasl_rt::from_word<" << e << ">(constant(" << next_word_ << " + i));\n";
      }
      refl_ << "uniform " << name << " " << next_word_ << " " << words << " " << ty.base << " " << ty.rows << " "
            << (ty.kind == Type::Scalar ? 1 : ty.cols) << "\n";
      next_word_ += words;
    }
    scopes_.front()[name] = s;
  }

  void parse_function(Type ret, std::string const& name) {
    Func f;
    f.name = name;
    f.ret = ret;
    expect("(");
    if (!is(")") && !(is("void") && peek(1).text == ")")) {
      for (;;) {
        Param p;
        for (;;) {
          if (accept("in")) continue;
          if (accept("uniform")) continue;
          if (accept("out")) {
            p.out = true;
            p.in = false;
            continue;
          }
          if (accept("inout")) {
            p.out = true;
            continue;
          }
          break;
        }
        p.type = parse_type();
        p.name = expect_id();
        p.type.array = parse_array_len();
        if (accept(":")) p.sem = parse_semantic();
        f.params.push_back(p);
        if (!accept(",")) break;
      }
    } else {
      accept("void");
    }
    expect(")");
    if (accept(":")) f.ret_sem = parse_semantic();
    if (accept(";")) {  // a prototype
      funcs_[name].push_back(f);
      return;
    }
    bool const entry = name == entry_;
    if (entry && have_entry_) fail("entry function '" + name + "' defined twice");
    funcs_[name].push_back(f);
    scopes_.emplace_back();
    std::ostringstream sig;
    sig << "  __host__ __device__ " << ret.cpp() << " f_" << name << "(";
    for (size_t i = 0; i < f.params.size(); ++i) {
      Param const& p = f.params[i];
      if (p.type.kind == Type::Sampler) fail("sampler parameters are not supported: use the global sampler");
      Sym s;
      s.type = p.type;
      s.code = "s_" + p.name;
      if (entry && !vs() && p.in && !p.out) bind_pixel_inputs(p, s);
      scopes_.back()[p.name] = s;
      if (i) sig << ", ";
      std::string const t = p.type.cpp();
      if (p.type.array)
        sig << t << " (" << (p.out ? "&" : "&") << "s_" << p.name << ")[" << p.type.array << "]";
      else if (p.out)
        sig << t << "& s_" << p.name;
      else
        sig << t << " s_" << p.name;
    }
    sig << ") const ";
    in_entry_ = entry;
    cur_ret_ = ret;
    std::string const body = block();
    in_entry_ = false;
    scopes_.pop_back();
    members_out_ << sig.str() << body << "\n";
    if (entry) {
      have_entry_ = true;
      entry_func_ = f;
    }
  }

  // the pixel inputs of an entry parameter, linked in order of appearance
  void bind_pixel_inputs(Param const& p, Sym& s) {
    if (p.type.kind == Type::Struct) {
      for (Member const& m : structs_[p.type.sname]) {
        if (!m.sem.present) fail("pixel input member '" + m.name + "' has no semantic");
        s.members_type[m.name] = m.type;
        if (m.sem.name == "SV_POSITION" || m.sem.name == "POSITION") continue;
        s.members_vary[m.name] = npsin_++;
      }
    } else if (p.sem.present && p.sem.name != "SV_POSITION" && p.sem.name != "POSITION") {
      s.vary = npsin_++;
    }
  }

  // ---- statements ------------------------------------------------------------
  std::string block() {
    expect("{");
    std::string out = "{\n";
    while (!accept("}")) {
      if (peek().kind == Token::End) fail("unterminated block");
      out += statement();
    }
    return out + "}\n";
  }

  std::string scoped(std::string (Translator::*fn)()) {
    scopes_.emplace_back();
    std::string s = (this->*fn)();
    scopes_.pop_back();
    return s;
  }

  std::string statement() {
    if (is("{")) return scoped(&Translator::block);
    if (accept(";")) return ";\n";
    if (accept("if")) {
      expect("(");
      Expr c = parse_expr();
      expect(")");
      std::string s = "if (" + c.code + ") " + scoped(&Translator::statement_block);
      if (accept("else")) s += "else " + scoped(&Translator::statement_block);
      return s;
    }
    if (accept("while")) {
      expect("(");
      Expr c = parse_expr();
      expect(")");
      return "while (" + c.code + ") " + scoped(&Translator::statement_block);
    }
    if (accept("do")) {
      std::string body = scoped(&Translator::statement_block);
      expect("while");
      expect("(");
      Expr c = parse_expr();
      expect(")");
      expect(";");
      return "do " + body + "while (" + c.code + ");\n";
    }
    if (accept("for")) {
      scopes_.emplace_back();
      expect("(");
      std::string init = ";";
      if (!accept(";")) {
        init = is_type_start() ? declaration() : parse_expr().code + ";";
        if (!is_type_start_decl_done_) expect(";");
        is_type_start_decl_done_ = false;
      }
      std::string cond, step;
      if (!is(";")) cond = parse_expr().code;
      expect(";");
      if (!is(")")) step = parse_expr().code;
      expect(")");
      std::string body = scoped(&Translator::statement_block);
      scopes_.pop_back();
      while (!init.empty() && (init.back() == '\n')) init.pop_back();
      return "for (" + init + " " + cond + "; " + step + ") " + body;
    }
    if (accept("switch")) {
      expect("(");
      Expr c = parse_expr();
      expect(")");
      expect("{");
      std::string s = "switch (" + c.code + ") {\n";
      scopes_.emplace_back();
      while (!accept("}")) {
        if (accept("case")) {
          Expr v = parse_cond();
          expect(":");
          s += "case " + v.code + ":\n";
        } else if (accept("default")) {
          expect(":");
          s += "default:\n";
        } else {
          if (peek().kind == Token::End) fail("unterminated switch");
          s += statement();
        }
      }
      scopes_.pop_back();
      return s + "}\n";
    }
    if (accept("return")) {
      if (accept(";")) return "return;\n";
      Expr e = parse_expr();
      expect(";");
      if (cur_ret_.numeric()) return "return sasl_rt::cast<" + cur_ret_.cpp() + ">(" + e.code + ");\n";
      return "return " + e.code + ";\n";
    }
    if (accept("break")) {
      expect(";");
      return "break;\n";
    }
    if (accept("continue")) {
      expect(";");
      return "continue;\n";
    }
    if (is("discard")) fail("discard is not supported");
    if (is_type_start()) {
      std::string d = declaration();
      if (!is_type_start_decl_done_) expect(";");
      is_type_start_decl_done_ = false;
      return d;
    }
    Expr e = parse_expr();
    expect(";");
    return e.code + ";\n";
  }
  bool is_type_start_decl_done_ = false;

  // a statement as the body of if / while / for: a block gets no extra scope
  std::string statement_block() { return is("{") ? block() : "{\n" + statement() + "}\n"; }

  std::string declaration() {
    while (accept("const") || accept("static") || accept("uniform")) {
    }
    Type ty = parse_type();
    if (ty.kind == Type::Sampler || ty.kind == Type::Void) fail("bad local variable type");
    std::string out;
    for (;;) {
      std::string const name = expect_id();
      Type vt = ty;
      vt.array = parse_array_len();
      if (accept(":")) parse_semantic();
      std::string const t = ty.cpp(), arr = vt.array ? "[" + std::to_string(vt.array) + "]" : "";
      if (accept("=")) {
        if (is("{")) {
          std::vector<Expr> items = init_list();
          if (vt.array) {
            out += t + " s_" + name + arr + " = {";
            for (size_t i = 0; i < items.size(); ++i)
              out += (i ? ", " : "") + (ty.kind == Type::Struct ? items[i].code : "sasl_rt::cast<" + t + ">(" + items[i].code + ")");
            out += "};\n";
          } else if (ty.numeric()) {
            out += t + " s_" + name + " = sasl_rt::make<" + t + ">(";
            for (size_t i = 0; i < items.size(); ++i) out += (i ? ", " : "") + items[i].code;
            out += ");\n";
          } else {
            fail("initialiser lists of structs are not supported");
          }
        } else {
          if (vt.array) fail("an array needs an initialiser list");
          Expr e = parse_assign();
          out += t + " s_" + name + " = " + (ty.numeric() ? "sasl_rt::cast<" + t + ">(" + e.code + ")" : e.code) + ";\n";
        }
      } else {
        out += t + " s_" + name + arr + "{};\n";
      }
      Sym s;
      s.type = vt;
      s.code = "s_" + name;
      scopes_.back()[name] = s;
      if (!accept(",")) break;
    }
    expect(";");
    is_type_start_decl_done_ = true;
    return out;
  }

  std::vector<Expr> init_list() {
    expect("{");
    std::vector<Expr> items;
    while (!accept("}")) {
      if (is("{")) fail("nested initialiser lists are not supported");
      items.push_back(parse_assign());
      if (!accept(",")) {
        expect("}");
        break;
      }
    }
    return items;
  }

  // ---- expressions -----------------------------------------------------------
  Expr parse_expr() {
    Expr e = parse_assign();
    while (accept(",")) {
      Expr r = parse_assign();
      e.code = "(" + e.code + ", " + r.code + ")";
      e.type = r.type;
      e.lvalue = false;
    }
    return e;
  }

  Expr parse_assign() {
    Expr l = parse_cond();
    static char const* const ops[] = {"=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="};
    for (char const* op : ops) {
      if (!is(op)) continue;
      int const line = peek().line;
      next();
      Expr r = parse_assign();
      if (!l.lvalue) throw SaslError{line, "the left side of '" + std::string(op) + "' is not assignable"};
      std::string const o = op;
      Expr out;
      out.type = l.type;
      if (l.multi) {
        std::string val = r.code;
        if (o != "=") {
          std::string const cur = "sasl_rt::swz<" + l.multi_idx + ">(" + l.multi_base + ")";
          std::string const bop = o.substr(0, o.size() - 1);
          val = bop == "/" ? "sasl_rt::div(" + cur + ", " + r.code + ")"
                : bop == "%" ? "sasl_rt::mod(" + cur + ", " + r.code + ")"
                             : "(" + cur + " " + bop + " " + r.code + ")";
        }
        out.code = "sasl_rt::swz_set<" + l.multi_idx + ">(" + l.multi_base + ", " + val + ")";
        return out;
      }
      bool const known = l.type.numeric() && !l.type.array;
      if (o == "=") {
        out.code = "(" + l.code + " = " + (known ? "sasl_rt::cast<" + l.type.cpp() + ">(" + r.code + ")" : r.code) + ")";
      } else if (o == "/=" || o == "%=") {
        std::string const fn = o == "/=" ? "sasl_rt::div" : "sasl_rt::mod";
        std::string const v = fn + "(" + l.code + ", " + r.code + ")";
        out.code = "(" + l.code + " = " + (known ? "sasl_rt::cast<" + l.type.cpp() + ">(" + v + ")" : v) + ")";
      } else {
        out.code = "(" + l.code + " " + o + " " + r.code + ")";
      }
      out.lvalue = false;
      return out;
    }
    return l;
  }

  Expr parse_cond() {
    Expr c = parse_binary(1);
    if (!accept("?")) return c;
    Expr a = parse_assign();
    expect(":");
    Expr b = parse_cond();
    Expr out;
    out.code = "(" + c.code + " ? " + a.code + " : " + b.code + ")";
    out.type = a.type;
    return out;
  }

  static int prec(std::string const& op) {
    static std::map<std::string, int> const p = {{"||", 1}, {"&&", 2}, {"|", 3},  {"^", 4},  {"&", 5},   {"==", 6},
                                                 {"!=", 6}, {"<", 7},  {">", 7},  {"<=", 7}, {">=", 7},  {"<<", 8},
                                                 {">>", 8}, {"+", 9},  {"-", 9},  {"*", 10}, {"/", 10},  {"%", 10}};
    auto it = p.find(op);
    return it == p.end() ? 0 : it->second;
  }

  static Type binary_type(Type const& a, Type const& b, std::string const& op) {
    Type t;
    if (!a.numeric() || !b.numeric()) return t;
    bool const cmp = op == "<" || op == ">" || op == "<=" || op == ">=" || op == "==" || op == "!=" || op == "&&" || op == "||";
    if (a.kind == Type::Matrix || b.kind == Type::Matrix) {
      t = a.kind == Type::Matrix ? a : b;
    } else if (a.kind == Type::Vector || b.kind == Type::Vector) {
      t.kind = Type::Vector;
      t.cols = std::max(a.kind == Type::Vector ? a.cols : 1, b.kind == Type::Vector ? b.cols : 1);
    } else {
      t.kind = Type::Scalar;
    }
    auto rank = [](std::string const& s) { return s == "double" ? 4 : s == "float" ? 3 : s == "uint" ? 2 : s == "int" ? 1 : 0; };
    if (cmp) {
      t.base = "bool";
    } else {
      int const r = std::max(std::max(rank(a.base), rank(b.base)), 1);
      t.base = r == 4 ? "double" : r == 3 ? "float" : r == 2 ? "uint" : "int";
    }
    t.array = 0;
    return t;
  }

  Expr parse_binary(int min_prec) {
    Expr l = parse_unary();
    for (;;) {
      if (peek().kind != Token::Punct) break;
      std::string const op = peek().text;
      int const p = prec(op);
      if (p == 0 || p < min_prec) break;
      next();
      Expr r = parse_binary(p + 1);
      Expr out;
      out.type = binary_type(l.type, r.type, op);
      if (op == "/")
        out.code = "sasl_rt::div(" + l.code + ", " + r.code + ")";
      else if (op == "%")
        out.code = "sasl_rt::mod(" + l.code + ", " + r.code + ")";
      else
        out.code = "(" + l.code + " " + op + " " + r.code + ")";
      l = out;
    }
    return l;
  }

  Expr parse_unary() {
    for (char const* op : {"-", "+", "!", "~"}) {
      if (accept(op)) {
        Expr e = parse_unary();
        e.code = std::string("(") + op + e.code + ")";
        e.lvalue = false;
        e.multi = false;
        e.vary = -1;
        if (std::string(op) == "!" && e.type.numeric()) e.type.base = "bool";
        return e;
      }
    }
    for (char const* op : {"++", "--"}) {
      if (accept(op)) {
        Expr e = parse_unary();
        if (!e.lvalue || e.multi) fail(std::string("operand of ") + op + " is not assignable");
        e.code = std::string("(") + op + e.code + ")";
        e.lvalue = false;
        return e;
      }
    }
    // a cast: '(' type ')' unary
    if (is("(") && peek(1).kind == Token::Id && peek(2).text == ")" &&
        (structs_.count(peek(1).text) || (type_from_name(peek(1).text).numeric()))) {
      next();
      Type t = parse_type();
      expect(")");
      Expr e = parse_unary();
      Expr out;
      out.type = t;
      out.code = t.kind == Type::Struct ? e.code : "sasl_rt::cast<" + t.cpp() + ">(" + e.code + ")";
      return out;
    }
    return parse_postfix(parse_primary());
  }

  static bool swizzle_index(char c, int& i) {
    switch (c) {
      case 'x': case 'r': i = 0; return true;
      case 'y': case 'g': i = 1; return true;
      case 'z': case 'b': i = 2; return true;
      case 'w': case 'a': i = 3; return true;
      default: return false;
    }
  }

  Expr parse_postfix(Expr e) {
    for (;;) {
      if (accept(".")) {
        std::string const name = expect_id();
        if (e.type.kind == Type::Struct && !e.type.array) {
          Member const* m = nullptr;
          for (Member const& mm : structs_[e.type.sname])
            if (mm.name == name) m = &mm;
          if (!m) fail("struct '" + e.type.sname + "' has no member '" + name + "'");
          Expr out;
          out.code = e.code + ".m_" + name;
          out.type = m->type;
          out.lvalue = e.lvalue;
          if (e.members_vary) {
            auto it = e.members_vary->find(name);
            if (it != e.members_vary->end()) {
              out.vary = it->second;
              out.vary_type = m->type;
            }
          }
          e = out;
          continue;
        }
        if (name.size() > 4) fail("bad swizzle '." + name + "'");
        std::vector<int> idx;
        for (char c : name) {
          int i;
          if (!swizzle_index(c, i)) fail("bad swizzle '." + name + "'");
          if (e.type.kind == Type::Vector && i >= e.type.cols) fail("swizzle '." + name + "' beyond the vector");
          if (e.type.kind == Type::Scalar && i > 0) fail("swizzle '." + name + "' of a scalar");
          idx.push_back(i);
        }
        std::string list;
        for (size_t k = 0; k < idx.size(); ++k) list += (k ? "," : "") + std::to_string(idx[k]);
        Expr out;
        out.type.kind = idx.size() == 1 ? Type::Scalar : Type::Vector;
        out.type.cols = static_cast<int>(idx.size());
        out.type.base = e.type.numeric() ? e.type.base : "";
        if (out.type.base.empty()) out.type.kind = Type::Unknown;
        std::set<int> uniq(idx.begin(), idx.end());
        if (idx.size() == 1) {
          out.code = "sasl_rt::comp<" + list + ">(" + e.code + ")";
          out.lvalue = e.lvalue;
        } else {
          out.code = "sasl_rt::swz<" + list + ">(" + e.code + ")";
          if (e.lvalue && uniq.size() == idx.size()) {
            out.lvalue = true;
            out.multi = true;
            out.multi_base = e.code;
            out.multi_idx = list;
          }
        }
        if (e.vary >= 0) {
          out.vary = e.vary;
          out.vary_type = e.vary_type;
          out.vary_wrap = e.vary_wrap;
          out.vary_wrap.push_back(idx.size() == 1 ? "sasl_rt::comp<" + list + ">" : "sasl_rt::swz<" + list + ">");
        }
        e = out;
        continue;
      }
      if (accept("[")) {
        Expr i = parse_expr();
        expect("]");
        Expr out;
        out.code = e.code + "[" + i.code + "]";
        out.lvalue = e.lvalue;
        if (e.type.array) {
          out.type = e.type;
          out.type.array = 0;
        } else if (e.type.kind == Type::Matrix) {
          out.type.kind = Type::Vector;
          out.type.base = e.type.base;
          out.type.cols = e.type.cols;
        } else if (e.type.kind == Type::Vector) {
          out.type.kind = Type::Scalar;
          out.type.base = e.type.base;
        }
        e = out;
        continue;
      }
      if (is("++") || is("--")) {
        if (!e.lvalue || e.multi) fail("operand of " + peek().text + " is not assignable");
        e.code = "(" + e.code + next().text + ")";
        e.lvalue = false;
        continue;
      }
      break;
    }
    return e;
  }

  std::vector<Expr> call_args() {
    expect("(");
    std::vector<Expr> args;
    if (accept(")")) return args;
    for (;;) {
      args.push_back(parse_assign());
      if (accept(")")) break;
      expect(",");
    }
    return args;
  }

  static std::string join(std::vector<Expr> const& a, size_t from = 0) {
    std::string s;
    for (size_t i = from; i < a.size(); ++i) s += (i > from ? ", " : "") + a[i].code;
    return s;
  }

  // the quad difference of a pixel input read directly
  std::string derivative(Expr const& a, char const* fn) {
    if (vs()) fail(std::string(fn) + " is a pixel-shader operation");
    if (a.vary < 0 || !in_entry_)
      fail(std::string(fn) + " applies to a pixel input read directly in the entry function "
                             "(the pipeline differences interpolated registers)");
    if (a.vary_type.kind == Type::Matrix || a.vary_type.array) fail("matrix and array pixel inputs are not supported");
    std::string code = "sasl_rt::from4<" + a.vary_type.cpp() + ">(" + fn + "(sasl_link(" + std::to_string(a.vary) + ")))";
    for (auto const& w : a.vary_wrap) code = w + "(" + code + ")";
    return code;
  }

  void use_sampler(Expr const& s, char const* fn) {
    if (!s.sampler) fail(std::string(fn) + ": the first argument must be a sampler");
    samplers_used_.insert(s.sampler_name);
    if (samplers_used_.size() > 1) fail("a stage samples through one sampler (slot 0)");
  }

  Expr intrinsic(std::string const& name, std::vector<Expr> const& a, bool& handled) {
    handled = true;
    Expr out;
    auto want = [&](size_t n) {
      if (a.size() != n) fail(name + " takes " + std::to_string(n) + " arguments");
    };
    Type f4;
    f4.kind = Type::Vector;
    f4.base = "float";
    f4.cols = 4;
    if (name == "ddx" || name == "ddy") {
      want(1);
      out.code = derivative(a[0], name.c_str());
      out.type = a[0].type;
      return out;
    }
    if (name == "tex2D") {
      want(2);
      use_sampler(a[0], "tex2D");
      if (vs()) fail("tex2D needs derivatives: use tex2Dlod in a vertex shader");
      std::string const dx = derivative(a[1], "ddx"), dy = derivative(a[1], "ddy");
      out.code = "sasl_tex2dgrad(sasl_rt::cast<sasl_rt::vec<float, 2>>(" + a[1].code + "), sasl_rt::cast<sasl_rt::vec<float, 2>>(" + dx +
                 "), sasl_rt::cast<sasl_rt::vec<float, 2>>(" + dy + "))";
      out.type = f4;
      return out;
    }
    if (name == "tex2Dgrad") {
      want(4);
      use_sampler(a[0], "tex2Dgrad");
      if (vs()) fail("tex2Dgrad is a pixel-shader lookup");
      out.code = "sasl_tex2dgrad(sasl_rt::cast<sasl_rt::vec<float, 2>>(" + a[1].code + "), sasl_rt::cast<sasl_rt::vec<float, 2>>(" +
                 a[2].code + "), sasl_rt::cast<sasl_rt::vec<float, 2>>(" + a[3].code + "))";
      out.type = f4;
      return out;
    }
    if (name == "tex2Dlod") {
      want(2);
      use_sampler(a[0], "tex2Dlod");
      out.code = "sasl_tex2dlod(sasl_rt::cast<sasl_rt::vec<float, 4>>(" + a[1].code + "))";
      out.type = f4;
      return out;
    }
    if (name == "tex2Dbias" || name == "tex2Dproj" || name == "texCUBE" || name == "texCUBElod" || name == "tex1D" ||
        name == "tex3D")
      fail(name + " is not implemented by the reference's shader bindings");
    static std::set<std::string> const generic = {
        "sqrt", "rsqrt", "exp",   "exp2",    "log",     "log2",      "log10", "sin",      "cos",   "tan",  "asin",
        "acos", "atan",  "sinh",  "cosh",    "tanh",    "floor",     "ceil",  "round",    "trunc", "frac", "saturate",
        "degrees", "radians", "pow", "fmod", "atan2", "step", "abs",  "sign",  "min",      "max",   "clamp", "lerp",
        "smoothstep", "dot", "cross", "length", "distance", "normalize", "reflect", "any", "all", "transpose", "mul"};
    if (generic.count(name)) {
      out.code = "sasl_rt::" + name + "(" + join(a) + ")";
      if (name == "dot" || name == "length" || name == "distance" || name == "any" || name == "all") {
        out.type.kind = Type::Scalar;
        out.type.base = (name == "any" || name == "all") ? "bool" : "float";
      } else if (name != "mul" && name != "transpose" && !a.empty() && a[0].type.numeric()) {
        out.type = a[0].type;
        if (out.type.base != "double" && name != "abs" && name != "sign" && name != "min" && name != "max" && name != "clamp")
          out.type.base = "float";
      }
      out.type.array = 0;
      return out;
    }
    handled = false;
    return out;
  }

  Expr parse_primary() {
    Token const t = peek();
    Expr e;
    if (t.kind == Token::Int || t.kind == Token::Float) {
      next();
      e.code = t.text;
      e.type.kind = Type::Scalar;
      e.type.base = t.kind == Token::Float ? "float" : (t.text.back() == 'u' ? "uint" : "int");
      return e;
    }
    if (accept("(")) {
      Expr in = parse_expr();
      expect(")");
      in.code = "(" + in.code + ")";
      return in;
    }
    if (t.kind != Token::Id) fail("unexpected '" + t.text + "'");
    if (t.text == "true" || t.text == "false") {
      next();
      e.code = t.text;
      e.type.kind = Type::Scalar;
      e.type.base = "bool";
      return e;
    }
    // constructors: floatN(...), floatRxC(...), float(x)
    Type const ct = type_from_name(t.text);
    if (ct.numeric() && peek(1).text == "(") {
      next();
      std::vector<Expr> args = call_args();
      e.type = ct;
      e.code = ct.kind == Type::Scalar ? "sasl_rt::cast<" + ct.cpp() + ">(" + join(args) + ")"
                                       : "sasl_rt::make<" + ct.cpp() + ">(" + join(args) + ")";
      return e;
    }
    if (peek(1).text == "(") {
      next();
      std::string const name = t.text;
      std::vector<Expr> args = call_args();
      auto f = funcs_.find(name);
      if (f != funcs_.end()) {
        Func const* pick = nullptr;
        for (Func const& fn : f->second)
          if (fn.params.size() == args.size()) pick = &fn;
        if (!pick) throw SaslError{t.line, "no overload of '" + name + "' takes " + std::to_string(args.size()) + " arguments"};
        if (name == entry_) throw SaslError{t.line, "the entry function cannot be called"};
        for (size_t i = 0; i < args.size(); ++i)
          if (pick->params[i].out && !args[i].lvalue) throw SaslError{t.line, "argument " + std::to_string(i + 1) + " of '" + name + "' must be assignable"};
        e.code = "f_" + name + "(" + join(args) + ")";
        e.type = pick->ret;
        return e;
      }
      bool handled = false;
      e = intrinsic(name, args, handled);
      if (!handled) throw SaslError{t.line, "unknown function '" + name + "'"};
      return e;
    }
    next();
    Sym const* s = lookup(t.text);
    if (!s) throw SaslError{t.line, "unknown name '" + t.text + "'"};
    e.type = s->type;
    if (s->kind == Sym::Sampler) {
      e.sampler = true;
      e.sampler_name = t.text;
      e.code = "0";
      return e;
    }
    e.code = s->code;
    e.lvalue = s->kind == Sym::Local || s->kind == Sym::Uniform;
    if (in_entry_ && s->vary >= 0) {
      e.vary = s->vary;
      e.vary_type = s->type;
    }
    if (in_entry_ && !s->members_vary.empty()) {
      e.members_vary = &s->members_vary;
      e.members_type = &s->members_type;
    }
    return e;
  }

  // ---- the class ---------------------------------------------------------------
  void io_items(Type const& t, Semantic const& sem, std::string const& path, std::vector<IoItem>& out, bool input) {
    if (t.kind == Type::Struct) {
      for (Member const& m : structs_[t.sname]) {
        if (m.type.kind == Type::Struct) throw SaslError{0, "nested structs in the stage interface are not supported"};
        io_items(m.type, m.sem, path + ".m_" + m.name, out, input);
      }
      return;
    }
    if (!sem.present) throw SaslError{0, std::string("a stage ") + (input ? "input" : "output") + " (" + path + ") has no semantic"};
    if (t.kind == Type::Matrix || t.array || !t.numeric())
      throw SaslError{0, "stage inputs and outputs must be scalars or vectors (" + path + ")"};
    out.push_back({sem, t, path});
  }

  void emit(std::string& source, std::string& reflection) {
    Func const& f = entry_func_;
    std::vector<IoItem> ins, outs;
    for (size_t i = 0; i < f.params.size(); ++i) {
      Param const& p = f.params[i];
      std::string const path = "a" + std::to_string(i);
      if (p.in) io_items(p.type, p.sem, path, ins, true);
      if (p.out) io_items(p.type, p.sem, path, outs, false);
    }
    if (f.ret.kind != Type::Void) io_items(f.ret, f.ret_sem, "r", outs, false);

    std::ostringstream w, rf;
    rf << "stage " << (vs() ? "vertex" : "pixel") << "\nentry " << entry_ << "\nclass " << cls_ << "\n";
    w << "  __host__ __device__ " << (vs() ? "void shader_prog(salvia_gb300::vs_input const& sg_in, salvia_gb300::vs_output& sg_out) const {\n"
                                           : "bool shader_prog(salvia_gb300::vs_output const& sg_in, salvia_gb300::ps_output& sg_out) const {\n");
    w << uniform_loads_.str();
    for (size_t i = 0; i < f.params.size(); ++i) {
      Param const& p = f.params[i];
      w << "    " << p.type.cpp() << " a" << i << (p.type.array ? "[" + std::to_string(p.type.array) + "]" : "") << "{};\n";
    }
    int reg = 0, link = 0;
    for (IoItem const& it : ins) {
      bool const position = it.sem.name == "SV_POSITION" || it.sem.name == "POSITION";
      if (vs()) {
        if (reg >= SG_MAX_VS_INPUTS) throw SaslError{0, "more than SG_MAX_VS_INPUTS vertex inputs"};
        w << "    " << it.path << " = sasl_rt::from4<" << it.type.cpp() << ">(sg_in.attribute(" << reg << "));\n";
        rf << "input " << it.sem.name << " " << it.sem.index << " " << reg << " " << it.type.comps() << "\n";
        ++reg;
      } else if (position) {
        w << "    " << it.path << " = sasl_rt::from4<" << it.type.cpp() << ">(sg_in.position);\n";
        rf << "input " << it.sem.name << " " << it.sem.index << " -1 " << it.type.comps() << "\n";
      } else {
        if (link >= SG_MAX_VARYINGS)
          throw SaslError{0, "more than " + std::to_string(SG_MAX_VARYINGS) + " pixel inputs besides the position"};
        w << "    " << it.path << " = sasl_rt::from4<" << it.type.cpp() << ">(sasl_rt::varying(sg_in, sasl_link(" << link << ")));\n";
        rf << "input " << it.sem.name << " " << it.sem.index << " " << link << " " << it.type.comps() << "\n";
        ++link;
      }
    }
    w << "    " << (f.ret.kind != Type::Void ? f.ret.cpp() + " r = " : "") << "f_" << entry_ << "(";
    for (size_t i = 0; i < f.params.size(); ++i) w << (i ? ", " : "") << "a" << i;
    w << ");\n";
    int varyings = 0;
    bool have_pos = false;
    std::set<int> targets;
    for (IoItem const& it : outs) {
      std::string const& n = it.sem.name;
      if (vs()) {
        if (n == "SV_POSITION" || n == "POSITION") {
          if (have_pos) throw SaslError{0, "two position outputs"};
          have_pos = true;
          w << "    sg_out.position = sasl_rt::to4(" << it.path << ");\n";
          rf << "output " << n << " " << it.sem.index << " -1 " << it.type.comps() << "\n";
        } else {
          if (varyings >= SG_MAX_VARYINGS)
            throw SaslError{0, "more than " + std::to_string(SG_MAX_VARYINGS) + " vertex outputs besides the position"};
          w << "    sg_out.attribute(" << varyings << ") = sasl_rt::to4(" << it.path << ");\n";
          rf << "output " << n << " " << it.sem.index << " " << varyings << " " << it.type.comps() << "\n";
          ++varyings;
        }
      } else {
        if (n != "COLOR" && n != "SV_TARGET") throw SaslError{0, "pixel output semantic " + n + " is not supported"};
        if (it.sem.index < 0 || it.sem.index >= SG_MAX_COLOR_TARGETS || !targets.insert(it.sem.index).second)
          throw SaslError{0, "bad or repeated colour target " + std::to_string(it.sem.index)};
        w << "    sg_out.color[" << it.sem.index << "] = sasl_rt::to4(" << it.path << ");\n";
        rf << "output " << n << " " << it.sem.index << " " << it.sem.index << " " << it.type.comps() << "\n";
      }
    }
    if (vs() && !have_pos) throw SaslError{0, "the vertex shader writes no SV_Position"};
    if (vs()) rf << "varyings " << varyings << "\n";
    w << (vs() ? "  }\n" : "    return true;\n  }\n");

    std::ostringstream s;
    s << "// SASL " << (vs() ? "vertex" : "pixel") << " shader '" << entry_ << "' as a shader module (sg_sasl_translate)\n"
      << "#include <salvia_gb300/sasl_rt.cuh>\n\nnamespace sasl_" << cls_ << " {\n"
      << structs_out_.str() << "struct " << cls_ << " : salvia_gb300::" << (vs() ? "vertex_shader" : "pixel_shader") << " {\n";
    if (!vs()) {
      s << "  // the varying register of pixel input k (constant word 47, three bits an input)\n"
        << "  __host__ __device__ int sasl_link(int k) const {\n"
        << "    uint32_t const r = (sasl_rt::bits(constant(47)) >> (3 * k)) & 7u;\n"
        << "    int const g = r ? static_cast<int>(r) - 1 : k;\n"
        << "    return g < SG_MAX_VARYINGS ? g : 0;\n  }\n"
        << "  __host__ __device__ sasl_rt::vec<float, 4> sasl_tex2dgrad(sasl_rt::vec<float, 2> uv, sasl_rt::vec<float, 2> dx,\n"
        << "                                                          sasl_rt::vec<float, 2> dy) const {\n"
        << "    salvia_gb300::vec4 const c = sample_grad(uv.v[0], uv.v[1], dx.v[0], dx.v[1], dy.v[0], dy.v[1]);\n"
        << "    return sasl_rt::make<sasl_rt::vec<float, 4>>(c.x, c.y, c.z, c.w);\n  }\n";
    }
    s << "  // sampler::sample_2d_lod(coord.xy, coord.w) (sampler_api.cpp tex2Dlod)\n"
      << "  __host__ __device__ sasl_rt::vec<float, 4> sasl_tex2dlod(sasl_rt::vec<float, 4> c) const {\n"
      << "    salvia_gb300::vec4 const t = sample(c.v[0], c.v[1], c.v[3]);\n"
      << "    return sasl_rt::make<sasl_rt::vec<float, 4>>(t.x, t.y, t.z, t.w);\n  }\n"
      << members_out_.str() << w.str() << "};\n}  // namespace sasl_" << cls_ << "\n\nusing " << cls_ << " = sasl_" << cls_
      << "::" << cls_ << ";\n"
      << (vs() ? "SALVIA_GB300_VERTEX_SHADER(" : "SALVIA_GB300_PIXEL_SHADER(") << cls_ << ")\n";
    source = s.str();
    reflection = rf.str() + refl_.str() + "words " + std::to_string(next_word_) + "\n";
  }
};

char* dup(std::string const& s) {
  char* p = static_cast<char*>(std::malloc(s.size() + 1));
  if (p) std::memcpy(p, s.c_str(), s.size() + 1);
  return p;
}

bool valid_class_name(char const* c) {
  if (!c || !*c || !(std::isalpha(static_cast<unsigned char>(*c)) || *c == '_')) return false;
  for (; *c; ++c)
    if (!(std::isalnum(static_cast<unsigned char>(*c)) || *c == '_')) return false;
  return true;
}

}  // namespace

extern "C" int32_t sg_sasl_translate(const char* source, uint32_t language, const char* entry, const char* class_name,
                                     char** out_source, char** out_reflection, char** out_log) {
  if (out_source) *out_source = nullptr;
  if (out_reflection) *out_reflection = nullptr;
  if (out_log) *out_log = nullptr;
  if (!source || !out_source || !out_reflection || !valid_class_name(class_name)) return SG_INVALID_PARAMETER;
  try {
    Translator t(source, static_cast<int>(language), entry ? entry : "", class_name);
    std::string src, refl;
    t.run(src, refl);
    *out_source = dup(src);
    *out_reflection = dup(refl);
    if (!*out_source || !*out_reflection) {
      std::free(*out_source);
      std::free(*out_reflection);
      *out_source = *out_reflection = nullptr;
      return SG_OUT_OF_MEMORY;
    }
    return SG_OK;
  } catch (SaslError const& e) {
    if (out_log) *out_log = dup((e.line ? "line " + std::to_string(e.line) + ": " : std::string()) + e.msg + "\n");
    return SG_INVALID_PARAMETER;
  }
}

extern "C" void sg_sasl_free(char* p) { std::free(p); }
