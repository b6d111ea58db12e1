// PDB reader for the atomic (complex-atom) model of the SAXS path: the bodies
// the reference's calc_saxs builds from PDB files with
// parse_pdb::all_models_as_complex_atoms (resaxslib/src/parse_pdb.cpp:63-108,
// 309-363).  The record handling, the fixed-column field layout of ATOM/HETATM
// records and the atom-type tables (resaxslib/src/utils.cpp:200-317) define
// which bodies exist and which form factor each gets, so they are kept equal
// to the reference's; the code is this project's.
#include "rsx.h"
#include "rsx_host.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace {

// atom types (resaxslib/include/constants.hpp:37-59)
enum AtomType : unsigned { H, C, N, O, P, S, Zn, CH, CH2, CH3, NH, NH2, NH3, OH, OH2, SH };

const std::map<std::string, AtomType> &element_types()
{
    static const std::map<std::string, AtomType> m = {{"H", H}, {"C", C}, {"N", N}, {"O", O},
                                                      {"P", P}, {"S", S}, {"Zn", Zn}};
    return m;
}

// atom label -> complex group regardless of residue
const std::map<std::string, AtomType> &group_types()
{
    static const std::map<std::string, AtomType> m = {{"CH2", CH2}, {"CH3", CH3}, {"CA", CH},
                                                      {"CB", CH2},  {"CG", CH2},  {"CG2", CH3},
                                                      {"CD", CH2},  {"N", NH}};
    return m;
}

// (atom label, residue) -> complex group, overriding the two maps above
const std::map<std::pair<std::string, std::string>, AtomType> &residue_group_types()
{
    static const std::map<std::pair<std::string, std::string>, AtomType> m = {
        {{"CA", "GLY"}, CH2},  {{"CB", "ALA"}, CH3},  {{"CB", "ILE"}, CH},   {{"CB", "THR"}, CH},
        {{"CB", "VAL"}, CH},   {{"CG", "ASN"}, C},    {{"CG", "ASP"}, C},    {{"CG", "HIS"}, C},
        {{"CG", "LEU"}, CH},   {{"CG", "PHE"}, C},    {{"CG", "TRP"}, C},    {{"CG", "TYR"}, C},
        {{"CG1", "ILE"}, CH2}, {{"CG1", "VAL"}, CH3}, {{"CD", "GLN"}, C},    {{"CD", "GLU"}, C},
        {{"CD1", "ILE"}, CH3}, {{"CD1", "LEU"}, CH3}, {{"CD1", "PHE"}, CH},  {{"CD1", "TRP"}, CH},
        {{"CD1", "TYR"}, CH},  {{"CD2", "HIS"}, CH},  {{"CD2", "LEU"}, CH3}, {{"CD2", "PHE"}, CH},
        {{"CD2", "TYR"}, CH},  {{"CE", "LYS"}, CH2},  {{"CE", "MET"}, CH3},  {{"CE1", "HIS"}, CH},
        {{"CE1", "PHE"}, CH},  {{"CE1", "TYR"}, CH},  {{"CE2", "PHE"}, CH},  {{"CE2", "TYR"}, CH},
        {{"CE3", "TRP"}, CH},  {{"CZ", "PHE"}, CH},   {{"CZ2", "TRP"}, CH},  {{"CZ3", "TRP"}, CH},
        {{"N", "PRO"}, N},     {{"ND1", "HIS"}, NH},  {{"ND2", "ASN"}, NH2}, {{"NH1", "ARG"}, NH2},
        {{"NH2", "ARG"}, NH2}, {{"NE", "ARG"}, NH},   {{"NE1", "TRP"}, NH},  {{"NE2", "GLN"}, NH2},
        {{"NZ", "LYS"}, NH3},  {{"OG", "SER"}, OH},   {{"OG1", "THR"}, OH},  {{"OH", "TYR"}, OH},
        {{"SG", "CYS"}, SH}};
    return m;
}

// Strips `delim` characters from both ends.  A string made only of delimiter
// characters keeps all but its last character, as the reference's trim does
// (resaxslib/src/utils.cpp:319-336); this decides, for instance, that a blank
// two-column element field is " " rather than empty.
std::string trim(const std::string &s, const char *delim = " ")
{
    const auto p1 = s.find_first_not_of(delim);
    const auto p2 = s.find_last_not_of(delim);
    return s.substr(p1 == std::string::npos ? 0 : p1,
                    p2 == std::string::npos ? s.length() - 1 : p2 - p1 + 1);
}

void parse_atom(const char *line, std::vector<rsx_body> &out, int verbose)
{
    char rec[7] = {0}, name[5] = {0}, res[4] = {0}, elem[3] = {0}, charge[3] = {0};
    int atom_n = 0, res_n = 0;
    char alt = 0, chain = 0, icode = 0;
    float x = 0, y = 0, z = 0, occ = 0, bfac = 0;
    // columns 1-6 record, 7-11 serial, 13-16 name, 17 altLoc, 18-20 residue,
    // 22 chain, 23-26 residue number, 27 iCode, 31-54 xyz, 55-60 occupancy,
    // 61-66 B factor, 77-78 element, 79-80 charge
    std::sscanf(line, "%6c%5d%*1c%4c%1c%3c%*1c%1c%4d%1c%*3c%8f%8f%8f%6f%6f%*10c%2c%2c", rec,
                &atom_n, name, &alt, res, &chain, &res_n, &icode, &x, &y, &z, &occ, &bfac, elem,
                charge);
    const std::string label = trim(name), residue = trim(res);
    std::string element = trim(elem);
    if (element.empty())
        element = label.substr(0, 1);
    if (residue == "HOH") // waters are left to the implicit water layer
        return;
    if (alt != ' ' && alt != 'A') // first alternate location only
        return;
    AtomType t;
    const auto e = element_types().find(element);
    if (e != element_types().end()) {
        t = e->second;
    } else {
        if (verbose >= 1)
            std::cerr << "Missing form factor for element " << element << " in residue " << residue
                      << "(" << res_n << ") - using N instead" << std::endl;
        t = N;
    }
    if (t == H) // hydrogens enter through the complex groups
        return;
    const auto g = group_types().find(label);
    if (g != group_types().end())
        t = g->second;
    const auto sp = residue_group_types().find({label, residue});
    if (sp != residue_group_types().end())
        t = sp->second;
    rsx_body b{x, y, z, 0.f};
    const unsigned bits = t;
    std::memcpy(&b.w, &bits, 4);
    out.push_back(b);
}

// Models in file order: MODEL opens one, ENDMDL closes it, ATOM/HETATM outside
// a model opens a new one, END stops reading.  Lines are read 99 characters at
// most (the rest is skipped) and a last line with no newline is not read, as
// in the reference's istream::getline loop.
rsx_status read_models(const char *path, int verbose, std::vector<std::vector<rsx_body>> &models)
{
    if (!path)
        return rsx::fail(RSX_INVALID_ARG, "rsx_pdb: null path");
    std::ifstream f(path);
    if (!f.is_open())
        return rsx::fail(RSX_PDB_FILE_NOT_FOUND, std::string(path) + " file not found");
    bool in_model = false;
    std::string line;
    while (true) {
        std::getline(f, line);
        if (f.bad() || f.eof())
            break;
        if (line.size() > 99)
            line.resize(99);
        std::string head = line.substr(0, 6);
        head.resize(6, ' ');
        const std::string rec = trim(head);
        if (rec == "END") {
            break;
        } else if (rec == "ENDMDL") {
            in_model = false;
        } else if (rec == "MODEL") {
            models.emplace_back();
            in_model = true;
        } else if (rec == "ATOM" || rec == "HETATM") {
            if (!in_model) {
                models.emplace_back();
                in_model = true;
            }
            parse_atom(line.c_str(), models.back(), verbose);
        }
    }
    return RSX_OK;
}

} // namespace

extern "C" rsx_status rsx_pdb_count(const char *path, int *n_models, int *n_bodies)
{
    if (!n_models || !n_bodies)
        return rsx::fail(RSX_INVALID_ARG, "rsx_pdb_count: null output");
    std::vector<std::vector<rsx_body>> models;
    const rsx_status st = read_models(path, 0, models);
    if (st != RSX_OK)
        return st;
    size_t total = 0;
    for (const auto &m : models)
        total += m.size();
    *n_models = (int)models.size();
    *n_bodies = (int)total;
    return rsx::ok();
}

extern "C" rsx_status rsx_pdb_read(const char *path, int verbose, rsx_body *out, int cap_bodies,
                                   int *model_sizes, int max_models)
{
    if (!out || !model_sizes)
        return rsx::fail(RSX_INVALID_ARG, "rsx_pdb_read: null output");
    std::vector<std::vector<rsx_body>> models;
    const rsx_status st = read_models(path, verbose, models);
    if (st != RSX_OK)
        return st;
    if ((int)models.size() > max_models)
        return rsx::fail(RSX_INVALID_ARG, "rsx_pdb_read: more models than max_models");
    size_t k = 0;
    for (size_t m = 0; m < models.size(); ++m) {
        if (k + models[m].size() > (size_t)cap_bodies)
            return rsx::fail(RSX_INVALID_ARG, "rsx_pdb_read: more bodies than cap_bodies");
        model_sizes[m] = (int)models[m].size();
        std::memcpy(out + k, models[m].data(), models[m].size() * sizeof(rsx_body));
        k += models[m].size();
    }
    return rsx::ok();
}
