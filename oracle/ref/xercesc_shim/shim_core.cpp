// shim_core.cpp -- implementation of the Xerces-C API subset declared in
// xercesc/shim_core.hpp.  Oracle build infrastructure only.
#include "xercesc/shim_core.hpp"

#include <cstring>

#include "xml_sax.hpp"

namespace xercesc_shim {

static XMLCh *dup16(const char *s) {
    size_t n = s ? strlen(s) : 0;
    XMLCh *r = new XMLCh[n + 1];
    for (size_t i = 0; i < n; i++) r[i] = (XMLCh)(unsigned char)s[i];
    r[n] = 0;
    return r;
}

static XMLCh *dup16(const XMLCh *s) {
    size_t n = XMLString::stringLen(s);
    XMLCh *r = new XMLCh[n + 1];
    for (size_t i = 0; i < n; i++) r[i] = s[i];
    r[n] = 0;
    return r;
}

static std::u16string to16(const std::string &s) {
    std::u16string r;
    r.reserve(s.size());
    for (unsigned char c : s) r.push_back((XMLCh)c);
    return r;
}

XMLSize_t XMLString::stringLen(const XMLCh *const s) {
    if (!s) return 0;
    XMLSize_t n = 0;
    while (s[n]) n++;
    return n;
}

char *XMLString::transcode(const XMLCh *const s) {
    size_t n = stringLen(s);
    char *r = new char[n + 1];
    for (size_t i = 0; i < n; i++) r[i] = (char)(s[i] & 0xFF);
    r[n] = 0;
    return r;
}

XMLCh *XMLString::transcode(const char *const s) { return dup16(s); }

void XMLString::release(char **p) {
    delete[] *p;
    *p = nullptr;
}

void XMLString::release(XMLCh **p) {
    delete[] *p;
    *p = nullptr;
}

XMLException::XMLException(const char *msg) : msg_(dup16(msg)) {}
XMLException::XMLException(const XMLException &o) : msg_(dup16(o.msg_)) {}
XMLException::~XMLException() { delete[] msg_; }

SAXException::SAXException() : msg_(dup16("")) {}
SAXException::SAXException(const char *const msg) : msg_(dup16(msg)) {}
SAXException::SAXException(const XMLCh *const msg) : msg_(dup16(msg)) {}
SAXException::SAXException(const SAXException &o) : msg_(dup16(o.msg_)) {}
SAXException &SAXException::operator=(const SAXException &o) {
    if (this != &o) {
        delete[] msg_;
        msg_ = dup16(o.msg_);
    }
    return *this;
}
SAXException::~SAXException() { delete[] msg_; }

SAXParseException::SAXParseException(const char *msg, const char *systemId, XMLFileLoc line, XMLFileLoc col)
    : SAXException(msg), sys_(dup16(systemId)), line_(line), col_(col) {}
SAXParseException::SAXParseException(const SAXParseException &o)
    : SAXException(o), sys_(dup16(o.sys_)), line_(o.line_), col_(o.col_) {}
SAXParseException::~SAXParseException() { delete[] sys_; }

const XMLCh *Attributes::getValue(const XMLCh *const qName) const {
    std::u16string q(qName ? qName : u"");
    for (size_t i = 0; i < names_.size(); i++)
        if (names_[i] == q) return values_[i].c_str();
    return nullptr;
}

const XMLCh *Attributes::getValue(const char *const qName) const { return getValue(to16(qName).c_str()); }

void Attributes::add(const std::string &n, const std::string &v) {
    names_.push_back(to16(n));
    values_.push_back(to16(v));
}

namespace {
class Bridge : public nairn_xml::Handler {
public:
    explicit Bridge(DefaultHandler *h) : h_(h) {}
    void start_element(const std::string &name, const std::vector<nairn_xml::Attr> &attrs) override {
        Attributes a;
        for (const auto &x : attrs) a.add(x.name, x.value);
        std::u16string n = to16(name);
        h_->startElement(u"", n.c_str(), n.c_str(), a);
    }
    void end_element(const std::string &name) override {
        std::u16string n = to16(name);
        h_->endElement(u"", n.c_str(), n.c_str());
    }
    void characters(const std::string &text) override {
        std::u16string t = to16(text);
        h_->characters(t.c_str(), t.size());
    }
private:
    DefaultHandler *h_;
};
}  // namespace

void SAX2XMLReader::parse(const char *const systemId) {
    DefaultHandler dummy;
    Bridge b(content_ ? content_ : &dummy);
    std::string err;
    try {
        if (!nairn_xml::parse_file(systemId, b, &err)) throw XMLException(err.c_str());
    } catch (const nairn_xml::ParseError &pe) {
        SAXParseException e(pe.message.c_str(), systemId, (XMLFileLoc)pe.line, (XMLFileLoc)pe.column);
        if (errors_)
            errors_->fatalError(e);
        else
            throw e;
    }
}

}  // namespace xercesc_shim
