// shim_core.hpp -- the subset of the Xerces-C 3.x SAX2 API that NairnMPM's
// sources use, implemented over this project's own XML reader
// (nairn-mpm-fea_gb300/csrc/host/xml_sax.cpp).  Oracle build infrastructure only:
// it exists so the reference's unmodified sources compile and read XML here,
// where no Xerces library is installed.
//
// Uses in the reference: Common/Read_XML/CommonReadHandler.hpp:25-33 (includes),
// Common/System/CommonAnalysis.cpp:184-273 (reader set-up, parse, exceptions),
// Common/Exceptions/StrX.hpp (transcode for messages).  XMLCh is a 16-bit unit;
// transcode maps bytes 1:1 to units and back, which is lossless for any input.
#ifndef NAIRN_XERCES_SHIM_CORE
#define NAIRN_XERCES_SHIM_CORE

#include <cstddef>
#include <string>
#include <vector>

typedef char16_t XMLCh;
typedef size_t XMLSize_t;
typedef unsigned long long XMLFileLoc;

namespace xercesc_shim {

class XMLString {
public:
    static char *transcode(const XMLCh *const s);
    static XMLCh *transcode(const char *const s);
    static void release(char **p);
    static void release(XMLCh **p);
    static XMLSize_t stringLen(const XMLCh *const s);
};

class XMLException {
public:
    explicit XMLException(const char *msg);
    XMLException(const XMLException &o);
    virtual ~XMLException();
    const XMLCh *getMessage() const { return msg_; }
private:
    XMLCh *msg_;
};

class XMLPlatformUtils {
public:
    static void Initialize() {}
    static void Terminate() {}
};

class SAXException {
public:
    SAXException();
    explicit SAXException(const char *const msg);
    explicit SAXException(const XMLCh *const msg);
    SAXException(const SAXException &o);
    SAXException &operator=(const SAXException &o);
    virtual ~SAXException();
    const XMLCh *getMessage() const { return msg_; }
protected:
    XMLCh *msg_;
};

class SAXParseException : public SAXException {
public:
    SAXParseException(const char *msg, const char *systemId, XMLFileLoc line, XMLFileLoc col);
    SAXParseException(const SAXParseException &o);
    ~SAXParseException();
    const XMLCh *getSystemId() const { return sys_; }
    XMLFileLoc getLineNumber() const { return line_; }
    XMLFileLoc getColumnNumber() const { return col_; }
private:
    XMLCh *sys_;
    XMLFileLoc line_, col_;
};

class Attributes {
public:
    Attributes() {}
    XMLSize_t getLength() const { return names_.size(); }
    const XMLCh *getLocalName(const XMLSize_t i) const { return i < names_.size() ? names_[i].c_str() : nullptr; }
    const XMLCh *getQName(const XMLSize_t i) const { return getLocalName(i); }
    const XMLCh *getValue(const XMLSize_t i) const { return i < values_.size() ? values_[i].c_str() : nullptr; }
    const XMLCh *getValue(const XMLCh *const qName) const;
    const XMLCh *getValue(const char *const qName) const;
    // shim-internal
    void add(const std::string &n, const std::string &v);
private:
    std::vector<std::u16string> names_, values_;
};

class DefaultHandler {
public:
    virtual ~DefaultHandler() {}
    virtual void startElement(const XMLCh *const, const XMLCh *const, const XMLCh *const, const Attributes &) {}
    virtual void endElement(const XMLCh *const, const XMLCh *const, const XMLCh *const) {}
    virtual void characters(const XMLCh *const, const XMLSize_t) {}
    virtual void warning(const SAXParseException &) {}
    virtual void error(const SAXParseException &) {}
    virtual void fatalError(const SAXParseException &e) { throw e; }
};

class SAX2XMLReader {
public:
    SAX2XMLReader() : content_(nullptr), errors_(nullptr) {}
    virtual ~SAX2XMLReader() {}
    void setFeature(const XMLCh *const, const bool) {}
    void setContentHandler(DefaultHandler *h) { content_ = h; }
    void setErrorHandler(DefaultHandler *h) { errors_ = h; }
    void parse(const char *const systemId);
private:
    DefaultHandler *content_;
    DefaultHandler *errors_;
};

class XMLReaderFactory {
public:
    static SAX2XMLReader *createXMLReader() { return new SAX2XMLReader(); }
};

}  // namespace xercesc_shim

#define XERCES_CPP_NAMESPACE_USE using namespace xercesc_shim;

#endif
