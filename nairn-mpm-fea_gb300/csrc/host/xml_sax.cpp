// xml_sax.cpp -- see xml_sax.hpp.
#include "xml_sax.hpp"

#include <cstdio>
#include <cstring>
#include <map>

namespace nairn_xml {

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

bool is_name_char(char c) {
    return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_' ||
           c == ':' || c == '-' || c == '.' || (unsigned char)c >= 0x80;
}

void append_utf8(std::string &out, unsigned long cp) {
    if (cp < 0x80) {
        out += (char)cp;
    } else if (cp < 0x800) {
        out += (char)(0xC0 | (cp >> 6));
        out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
        out += (char)(0xE0 | (cp >> 12));
        out += (char)(0x80 | ((cp >> 6) & 0x3F));
        out += (char)(0x80 | (cp & 0x3F));
    } else {
        out += (char)(0xF0 | (cp >> 18));
        out += (char)(0x80 | ((cp >> 12) & 0x3F));
        out += (char)(0x80 | ((cp >> 6) & 0x3F));
        out += (char)(0x80 | (cp & 0x3F));
    }
}

class Parser {
public:
    Parser(const std::string &doc, Handler &h) : d_(doc), h_(h), p_(0) {}

    void run() {
        if (d_.size() >= 3 && (unsigned char)d_[0] == 0xEF && (unsigned char)d_[1] == 0xBB &&
            (unsigned char)d_[2] == 0xBF)
            p_ = 3;
        prolog();
        // Expand user-declared entities textually in the rest of the document,
        // so an entity may hold markup as well as text.
        if (!ents_.empty()) {
            std::string rest = expand_user_entities(d_.substr(p_));
            d_ = d_.substr(0, p_) + rest;
        }
        content();
    }

private:
    std::string d_;
    Handler &h_;
    size_t p_;
    std::map<std::string, std::string> ents_;

    [[noreturn]] void fail(const char *msg) {
        int line = 1, col = 1;
        for (size_t i = 0; i < p_ && i < d_.size(); i++) {
            if (d_[i] == '\n') {
                line++;
                col = 1;
            } else {
                col++;
            }
        }
        throw ParseError{msg, line, col};
    }

    bool starts(const char *s) const { return d_.compare(p_, strlen(s), s) == 0; }

    void skip_space() {
        while (p_ < d_.size() && is_space(d_[p_])) p_++;
    }

    void skip_past(const char *term, const char *err) {
        size_t q = d_.find(term, p_);
        if (q == std::string::npos) fail(err);
        p_ = q + strlen(term);
    }

    std::string read_name() {
        size_t s = p_;
        while (p_ < d_.size() && is_name_char(d_[p_])) p_++;
        if (p_ == s) fail("expected a name");
        return d_.substr(s, p_ - s);
    }

    std::string read_quoted_raw() {
        if (p_ >= d_.size() || (d_[p_] != '"' && d_[p_] != '\'')) fail("expected a quoted value");
        char q = d_[p_++];
        size_t e = d_.find(q, p_);
        if (e == std::string::npos) fail("unterminated quoted value");
        std::string v = d_.substr(p_, e - p_);
        p_ = e + 1;
        return v;
    }

    void doctype() {
        p_ += 9;  // "<!DOCTYPE"
        skip_space();
        read_name();
        // external id and anything else up to '[' or '>'
        while (p_ < d_.size() && d_[p_] != '[' && d_[p_] != '>') {
            if (d_[p_] == '"' || d_[p_] == '\'')
                read_quoted_raw();
            else
                p_++;
        }
        if (p_ >= d_.size()) fail("unterminated DOCTYPE");
        if (d_[p_] == '[') {
            p_++;
            for (;;) {
                skip_space();
                if (p_ >= d_.size()) fail("unterminated DOCTYPE internal subset");
                if (d_[p_] == ']') {
                    p_++;
                    break;
                }
                if (starts("<!--")) {
                    skip_past("-->", "unterminated comment");
                } else if (starts("<!ENTITY")) {
                    p_ += 8;
                    skip_space();
                    bool param = false;
                    if (p_ < d_.size() && d_[p_] == '%') {
                        param = true;
                        p_++;
                        skip_space();
                    }
                    std::string name = read_name();
                    skip_space();
                    if (p_ < d_.size() && (d_[p_] == '"' || d_[p_] == '\'')) {
                        std::string v = read_quoted_raw();
                        if (!param && !ents_.count(name)) ents_[name] = v;
                    }
                    skip_past(">", "unterminated ENTITY declaration");
                } else if (starts("<?")) {
                    skip_past("?>", "unterminated processing instruction");
                } else if (starts("<!")) {
                    // ELEMENT / ATTLIST / NOTATION: skip, honouring quotes
                    while (p_ < d_.size() && d_[p_] != '>') {
                        if (d_[p_] == '"' || d_[p_] == '\'')
                            read_quoted_raw();
                        else
                            p_++;
                    }
                    if (p_ >= d_.size()) fail("unterminated markup declaration");
                    p_++;
                } else {
                    p_++;  // parameter entity references and stray text
                }
            }
            skip_space();
        }
        if (p_ >= d_.size() || d_[p_] != '>') fail("unterminated DOCTYPE");
        p_++;
    }

    void prolog() {
        for (;;) {
            skip_space();
            if (starts("<?")) {
                skip_past("?>", "unterminated processing instruction");
            } else if (starts("<!--")) {
                skip_past("-->", "unterminated comment");
            } else if (starts("<!DOCTYPE")) {
                doctype();
            } else {
                return;
            }
        }
    }

    std::string expand_user_entities(const std::string &in) {
        std::string cur = in;
        for (int pass = 0; pass < 16; pass++) {
            std::string out;
            out.reserve(cur.size());
            bool changed = false;
            size_t i = 0;
            while (i < cur.size()) {
                if (cur[i] == '&') {
                    size_t semi = cur.find(';', i + 1);
                    if (semi != std::string::npos && semi - i < 128) {
                        std::string nm = cur.substr(i + 1, semi - i - 1);
                        auto it = ents_.find(nm);
                        if (it != ents_.end()) {
                            out += it->second;
                            i = semi + 1;
                            changed = true;
                            continue;
                        }
                    }
                }
                out += cur[i++];
            }
            cur.swap(out);
            if (!changed) break;
        }
        return cur;
    }

    // Decode predefined and numeric character references.
    std::string decode(const std::string &s, bool attribute) {
        std::string out;
        out.reserve(s.size());
        for (size_t i = 0; i < s.size(); i++) {
            char c = s[i];
            if (c == '&') {
                size_t semi = s.find(';', i + 1);
                if (semi == std::string::npos) fail("unterminated character reference");
                std::string r = s.substr(i + 1, semi - i - 1);
                if (r == "lt")
                    out += '<';
                else if (r == "gt")
                    out += '>';
                else if (r == "amp")
                    out += '&';
                else if (r == "quot")
                    out += '"';
                else if (r == "apos")
                    out += '\'';
                else if (r.size() > 1 && r[0] == '#') {
                    unsigned long cp = (r[1] == 'x') ? strtoul(r.c_str() + 2, nullptr, 16)
                                                     : strtoul(r.c_str() + 1, nullptr, 10);
                    append_utf8(out, cp);
                } else {
                    fail("reference to an undeclared entity");
                }
                i = semi;
            } else if (attribute && (c == '\t' || c == '\n' || c == '\r')) {
                out += ' ';
            } else {
                out += c;
            }
        }
        return out;
    }

    void content() {
        std::vector<std::string> stack;
        bool seen_root = false;
        std::string text;
        auto flush_text = [&]() {
            if (!text.empty()) {
                if (!stack.empty()) h_.characters(text);
                text.clear();
            }
        };
        while (p_ < d_.size()) {
            char c = d_[p_];
            if (c != '<') {
                size_t e = d_.find('<', p_);
                if (e == std::string::npos) e = d_.size();
                std::string raw = d_.substr(p_, e - p_);
                if (stack.empty()) {
                    for (char ch : raw)
                        if (!is_space(ch)) fail("text outside the root element");
                } else {
                    text += decode(raw, false);
                }
                p_ = e;
                continue;
            }
            if (starts("<!--")) {
                skip_past("-->", "unterminated comment");
                continue;
            }
            if (starts("<![CDATA[")) {
                p_ += 9;
                size_t e = d_.find("]]>", p_);
                if (e == std::string::npos) fail("unterminated CDATA section");
                text += d_.substr(p_, e - p_);
                p_ = e + 3;
                continue;
            }
            if (starts("<?")) {
                skip_past("?>", "unterminated processing instruction");
                continue;
            }
            flush_text();
            if (starts("</")) {
                p_ += 2;
                std::string nm = read_name();
                skip_space();
                if (p_ >= d_.size() || d_[p_] != '>') fail("malformed end tag");
                p_++;
                if (stack.empty() || stack.back() != nm) fail("mismatched end tag");
                stack.pop_back();
                h_.end_element(nm);
                continue;
            }
            // start tag
            p_++;
            if (stack.empty() && seen_root) fail("more than one root element");
            std::string nm = read_name();
            std::vector<Attr> attrs;
            bool empty = false;
            for (;;) {
                skip_space();
                if (p_ >= d_.size()) fail("unterminated start tag");
                if (d_[p_] == '>') {
                    p_++;
                    break;
                }
                if (starts("/>")) {
                    p_ += 2;
                    empty = true;
                    break;
                }
                std::string an = read_name();
                skip_space();
                if (p_ >= d_.size() || d_[p_] != '=') fail("expected '=' after attribute name");
                p_++;
                skip_space();
                std::string av = decode(read_quoted_raw(), true);
                attrs.push_back(Attr{an, av});
            }
            seen_root = true;
            stack.push_back(nm);
            h_.start_element(nm, attrs);
            if (empty) {
                stack.pop_back();
                h_.end_element(nm);
            }
        }
        if (!stack.empty()) fail("document ended inside an element");
        if (!seen_root) fail("no root element");
    }
};

}  // namespace

void parse_string(const std::string &doc, Handler &h) {
    Parser p(doc, h);
    p.run();
}

bool parse_file(const char *path, Handler &h, std::string *err) {
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        if (err) *err = std::string("cannot open ") + path;
        return false;
    }
    std::string doc;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), fp)) > 0) doc.append(buf, n);
    fclose(fp);
    parse_string(doc, h);
    return true;
}

}  // namespace nairn_xml
