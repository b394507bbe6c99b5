// xml_sax.hpp -- a small, dependency-free SAX-style XML reader.
//
// NairnMPM reads its input through a SAX2 event stream (element start with
// attributes, character data, element end); see Common/System/CommonAnalysis.cpp:184-273
// (CommonAnalysis::ReadFile) and Common/Read_XML/CommonReadHandler.cpp:48-360.
// This reader produces the same event stream for the XML subset NairnMPM input
// files use: the prolog (<?xml ...?>), comments, a DOCTYPE whose internal subset
// declares text entities (<!ENTITY name "value">, as in
// NairnMPM/input/XML_Input/TwoDisks.fmcmd:2-12), CDATA sections, elements with
// single- or double-quoted attributes, and the predefined and numeric character
// references.  It does no validation and no namespace processing.
#pragma once

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

namespace nairn_xml {

struct Attr {
    std::string name;
    std::string value;
};

// Event receiver.  Exceptions thrown by a callback propagate out of parse().
class Handler {
public:
    virtual ~Handler() {}
    virtual void start_element(const std::string &name, const std::vector<Attr> &attrs) = 0;
    virtual void end_element(const std::string &name) = 0;
    virtual void characters(const std::string &text) = 0;
};

// Raised for malformed input; carries the 1-based line and column.
struct ParseError {
    std::string message;
    int line;
    int column;
};

// Parse a whole document held in memory.  Throws ParseError on malformed XML.
void parse_string(const std::string &doc, Handler &h);

// Read a file and parse it.  Returns false (and leaves h untouched) when the
// file cannot be read.
bool parse_file(const char *path, Handler &h, std::string *err);

}  // namespace nairn_xml
