// Native input parsers (include/plk.h, "input formats"): character matrices
// (FASTA, relaxed PHYLIP, NEXUS DATA block) into the engine's state-set masks
// and Newick trees into its flat node arrays.  They restate the reference's
// matrix_parser::pars_fasta / pars_relaxed_phylip / pars_nexus
// (src/matrix_parser.cpp:27-225) and tree::tree_file_parser
// (src/tree.cpp:69-237) on in-memory text, so a caller can go from files to
// plk_set_alignment / plk_set_tree without the reference's object graph.
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "plk_internal.h"

using namespace plk;

namespace {

// IUPAC nucleotide codes on the engine's DNA state order A=0, G=1, C=2, T=3
// (the reference's dna alphabet); -1 = not part of the alphabet
void dna_alphabet(int32_t* table) {
    for (int c = 0; c < 256; ++c) table[c] = -1;
    const struct { char c; int mask; } codes[] = {
        {'A', 1}, {'G', 2}, {'C', 4}, {'T', 8}, {'-', 0}, {'.', 0}, {'R', 3}, {'Y', 12}, {'S', 6}, {'W', 9},
        {'K', 10}, {'M', 5}, {'B', 14}, {'D', 11}, {'H', 13}, {'V', 7}, {'N', 15}};
    for (const auto& e : codes) {
        table[(unsigned char)e.c] = e.mask;
        if (std::isalpha((unsigned char)e.c)) table[std::tolower((unsigned char)e.c)] = e.mask;
    }
}

struct Matrix {
    std::vector<std::string> names;
    std::vector<std::vector<uint32_t>> rows;
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// src/matrix_parser.cpp pars_fasta: '>' starts a name that runs to the end of
// the line (blanks dropped); every other non-blank character is one cell,
// characters outside the alphabet giving an empty cell; a name with no cells
// after it is dropped, as the reference drops empty rows
void parse_fasta(const char* t, size_t n, const int32_t* alpha, Matrix* m) {
    char mode = 'n';
    std::string name, row_name;
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        const char c = t[i];
        if (c == '>') {
            mode = 't';
        } else if (mode == 't' && (c == '\n' || c == '\r')) {
            if (!row.empty()) {
                m->names.push_back(row_name);
                m->rows.push_back(row);
            }
            row.clear();
            row_name = name;
            name.clear();
            mode = 's';
        } else if (c != '\n' && c != '\r' && c != '\t' && c != ' ') {
            if (mode == 't') name += c;
            else if (mode == 's') {
                const int32_t v = alpha[(unsigned char)c];
                row.push_back(v < 0 ? 0u : (uint32_t)v);
            }
        }
    }
    if (!row.empty()) {
        m->names.push_back(row_name);
        m->rows.push_back(row);
    }
}

// cells of one matrix row in the PHYLIP / NEXUS readers: characters outside
// the alphabet are skipped
void add_cell(std::vector<uint32_t>& row, const int32_t* alpha, char c) {
    const int32_t v = alpha[(unsigned char)c];
    if (v >= 0) row.push_back((uint32_t)v);
}

// src/matrix_parser.cpp pars_relaxed_phylip: "n_taxa n_char" header, then per
// line a name up to the first blank and the cells up to the end of the line
bool parse_phylip(const char* t, size_t n, const int32_t* alpha, Matrix* m, std::string* err) {
    size_t i = 0;
    auto read_int = [&](long* out) -> bool {
        while (i < n && is_space(t[i])) ++i;
        size_t j = i;
        while (j < n && std::isdigit((unsigned char)t[j])) ++j;
        if (j == i) return false;
        *out = std::strtol(std::string(t + i, t + j).c_str(), nullptr, 10);
        i = j;
        return true;
    };
    long n_taxa = 0, n_char = 0;
    if (!read_int(&n_taxa) || !read_int(&n_char)) {
        *err = "PHYLIP header needs the numbers of taxa and characters";
        return false;
    }
    while (i < n && t[i] != '\n') ++i;
    while (i < n) {
        while (i < n && is_space(t[i])) ++i;
        if (i >= n) break;
        std::string name;
        while (i < n && !is_space(t[i])) name += t[i++];
        std::vector<uint32_t> row;
        while (i < n && t[i] != '\n' && t[i] != '\r') add_cell(row, alpha, t[i++]);
        m->names.push_back(name);
        m->rows.push_back(row);
    }
    if ((long)m->rows.size() != n_taxa) {
        *err = "PHYLIP header says " + std::to_string(n_taxa) + " taxa, the matrix has " + std::to_string(m->rows.size());
        return false;
    }
    return true;
}

// src/matrix_parser.cpp pars_nexus: keywords ntax= / nchar= (case-insensitive)
// before "matrix"; then rows of a name and cells up to the end of the line,
// ended by ';'
bool parse_nexus(const char* t, size_t n, const int32_t* alpha, Matrix* m, std::string* err) {
    std::string word;
    size_t i = 0;
    long n_taxa = 0;
    bool found = false;
    auto lower = [](std::string s) {
        for (char& c : s) c = (char)std::tolower((unsigned char)c);
        return s;
    };
    for (; i < n; ++i) {
        const char c = t[i];
        if (c == ' ' || c == ';' || c == '=' || c == '\n' || c == '\r' || c == '\t') {
            if (word.empty()) continue;
            const std::string w = lower(word);
            word.clear();
            if (w == "matrix") {
                found = true;
                ++i;
                break;
            }
            if (w == "ntax") {
                while (i < n && (t[i] == '=' || t[i] == ' ')) ++i;
                n_taxa = std::strtol(t + i, nullptr, 10);
            }
        } else {
            word += c;
        }
    }
    if (!found) {
        *err = "NEXUS text has no MATRIX command";
        return false;
    }
    while (i < n) {
        while (i < n && is_space(t[i])) ++i;
        if (i >= n || t[i] == ';') break;
        std::string name;
        while (i < n && !is_space(t[i]) && t[i] != ';') name += t[i++];
        std::vector<uint32_t> row;
        while (i < n && t[i] != '\n' && t[i] != '\r' && t[i] != ';') add_cell(row, alpha, t[i++]);
        m->names.push_back(name);
        m->rows.push_back(row);
    }
    if (n_taxa > 0 && (long)m->rows.size() != n_taxa) {
        *err = "NEXUS ntax says " + std::to_string(n_taxa) + " taxa, the matrix has " + std::to_string(m->rows.size());
        return false;
    }
    return true;
}

// ---- Newick (src/tree.cpp:69-237) ------------------------------------------
struct TNode {
    TNode* parent = nullptr;
    TNode* left = nullptr;
    TNode* right = nullptr;
    std::string label;
    bool has_label = false;
    double bl = 0.0;
};

struct Tree {
    std::vector<std::unique_ptr<TNode>> pool;
    TNode* make(TNode* parent) {
        pool.emplace_back(new TNode());
        pool.back()->parent = parent;
        return pool.back().get();
    }
};

// one tree: '(' opens a left child, ',' a right child (a third child pushes
// the two existing ones under a new zero-length node), ')' climbs, ':' starts
// a branch length (read as atof reads it), '[...]' is a comment, quotes
// enclose a label; ';' ends the tree.  Blanks are skipped everywhere (the
// reference reads the file with whitespace-skipping stream extraction).
bool parse_newick_tree(const char* t, size_t n, Tree* tree, TNode** root_out, std::string* err) {
    TNode* root = tree->make(nullptr);
    TNode* present = root;
    std::string label, bl_text;
    char mode = 's';
    auto flush = [&](TNode* node) {
        if (!label.empty()) {
            node->label = label;
            node->has_label = true;
            label.clear();
        }
        if (!bl_text.empty()) {
            node->bl = std::atof(bl_text.c_str());
            bl_text.clear();
        }
    };
    bool ended = false;
    for (size_t i = 0; i < n && !ended; ++i) {
        const char c = t[i];
        if (is_space(c)) continue;
        if (c == '[') {
            int depth = 1;
            while (++i < n && depth > 0) {
                if (t[i] == '[') ++depth;
                else if (t[i] == ']') --depth;
            }
            --i;
            continue;
        }
        switch (c) {
            case '(':
                mode = 'l';
                present->left = tree->make(present);
                present = present->left;
                label.clear();
                break;
            case ',':
                mode = 'l';
                flush(present);
                present = present->parent;
                if (!present) { *err = "unbalanced ',' in Newick text"; return false; }
                if (!present->right) {
                    present->right = tree->make(present);
                    present = present->right;
                } else {
                    TNode* extra = tree->make(present);
                    extra->left = present->left;
                    extra->right = present->right;
                    extra->left->parent = extra;
                    extra->right->parent = extra;
                    present->left = extra;
                    present->right = tree->make(present);
                    present = present->right;
                }
                break;
            case ')':
                mode = 'l';
                flush(present);
                present = present->parent;
                if (!present) { *err = "unbalanced ')' in Newick text"; return false; }
                break;
            case ':':
                mode = 'b';
                break;
            case ';':
                flush(present);
                if (!present->right && present->left && present->has_label) {
                    TNode* r = tree->make(present);
                    r->label = present->label;
                    r->has_label = true;
                    r->bl = present->bl;
                    present->right = r;
                    present->has_label = false;
                    present->label.clear();
                    present->bl = 0.0;
                }
                ended = true;
                break;
            default:
                if (mode == 'b') {
                    bl_text += c;
                } else if (mode == 'l') {
                    if (label.empty() && (c == '\'' || c == '"')) {
                        // blanks are dropped everywhere, quoted labels included
                        while (++i < n && t[i] != c)
                            if (!is_space(t[i])) label += t[i];
                    } else {
                        label += c;
                    }
                }
        }
    }
    if (!ended) { *err = "Newick text has no ';'"; return false; }
    *root_out = root;
    return true;
}

void post_order(TNode* v, std::vector<TNode*>* out) {
    if (!v) return;
    post_order(v->left, out);
    post_order(v->right, out);
    out->push_back(v);
}

}  // namespace

extern "C" {

plk_status plk_parse_alignment(const char* text, size_t len, int format, const int32_t* alphabet, int* n_taxa_out,
                               int* n_sites_out, uint32_t* masks_out, char* names_out, size_t names_cap) {
    if (!text || !n_taxa_out || !n_sites_out) return report_error(PLK_ERR_ARG, "bad arguments to plk_parse_alignment");
    int32_t dna[256];
    if (!alphabet) {
        dna_alphabet(dna);
        alphabet = dna;
    }
    Matrix m;
    std::string err;
    bool ok = true;
    if (format == PLK_FORMAT_FASTA) parse_fasta(text, len, alphabet, &m);
    else if (format == PLK_FORMAT_PHYLIP) ok = parse_phylip(text, len, alphabet, &m, &err);
    else if (format == PLK_FORMAT_NEXUS) ok = parse_nexus(text, len, alphabet, &m, &err);
    else return report_error(PLK_ERR_ARG, "unknown alignment format");
    if (!ok) return report_error(PLK_ERR_ARG, err);
    if (m.rows.empty()) return report_error(PLK_ERR_ARG, "no sequences in the alignment text");
    size_t n_sites = 0;
    for (const auto& r : m.rows) n_sites = std::max(n_sites, r.size());
    *n_taxa_out = (int)m.rows.size();
    *n_sites_out = (int)n_sites;
    if (masks_out) {
        // empty cells (gaps, unknown characters, short rows) allow every state,
        // as treeator sets them (src/treeator.cpp:463-466)
        uint32_t all = 0;
        for (int c = 0; c < 256; ++c)
            if (alphabet[c] > 0) all |= (uint32_t)alphabet[c];
        for (size_t t = 0; t < m.rows.size(); ++t)
            for (size_t s = 0; s < n_sites; ++s) {
                const uint32_t v = s < m.rows[t].size() ? m.rows[t][s] : 0u;
                masks_out[t * n_sites + s] = v ? v : all;
            }
    }
    if (names_out) {
        size_t need = 0;
        for (const auto& nm : m.names) need += nm.size() + 1;
        if (need > names_cap) return report_error(PLK_ERR_ARG, "names buffer too small: " + std::to_string(need) + " bytes needed");
        size_t off = 0;
        for (const auto& nm : m.names) {
            std::memcpy(names_out + off, nm.c_str(), nm.size() + 1);
            off += nm.size() + 1;
        }
    }
    return PLK_OK;
}

plk_status plk_parse_newick(const char* text, size_t len, int n_taxa, const char* names, int* n_nodes_out,
                            int* left, int* right, double* bl) {
    if (!text || !n_nodes_out) return report_error(PLK_ERR_ARG, "bad arguments to plk_parse_newick");
    Tree tree;
    TNode* root = nullptr;
    std::string err;
    if (!parse_newick_tree(text, len, &tree, &root, &err)) return report_error(PLK_ERR_ARG, err);
    std::vector<TNode*> order;
    post_order(root, &order);
    const int n = (int)order.size();
    *n_nodes_out = n;
    if (!left && !right && !bl) return PLK_OK;
    if (!left || !right || !bl) return report_error(PLK_ERR_ARG, "left, right and bl are all needed");
    // tips first (row of their name, or order of appearance), internal nodes
    // after them in post-order
    std::map<std::string, int> row_of;
    if (names) {
        const char* p = names;
        for (int i = 0; i < n_taxa; ++i) {
            row_of[p] = i;
            p += std::strlen(p) + 1;
        }
    }
    std::map<const TNode*, int> id;
    int n_tips = 0;
    for (const TNode* v : order)
        if (!v->left && !v->right) ++n_tips;
    if (names && n_tips != n_taxa)
        return report_error(PLK_ERR_ARG, "tree has " + std::to_string(n_tips) + " tips, " + std::to_string(n_taxa) + " names given");
    int next_tip = 0, next_int = n_tips;
    for (const TNode* v : order) {
        if (!v->left && !v->right) {
            if (names) {
                auto it = row_of.find(v->label);
                if (it == row_of.end()) return report_error(PLK_ERR_ARG, "tip label '" + v->label + "' is not a taxon name");
                id[v] = it->second;
            } else {
                id[v] = next_tip++;
            }
        } else {
            id[v] = next_int++;
        }
    }
    std::vector<char> seen(n, 0);
    for (const TNode* v : order) {
        const int k = id[v];
        if (seen[k]) return report_error(PLK_ERR_ARG, "two tips carry the label '" + v->label + "'");
        seen[k] = 1;
        left[k] = v->left ? id[v->left] : -1;
        right[k] = v->right ? id[v->right] : -1;
        bl[k] = v->bl;
    }
    return PLK_OK;
}

}  // extern "C"
