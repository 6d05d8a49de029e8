// Marching-cubes tables, identical in content to the reference's
// (GPU/MarchingCubesHelper.cpp:3-577, the public Lorensen-Cline / Bourke 1994
// tables), because MC case indices and triangle order must match bit for
// bit.  The encoding is this project's own:
//   kTriPacked[c]  cut-edge list of case c, one 4-bit edge id per nibble from
//                  the least significant end, three per triangle, unused
//                  nibbles = 0xF;
//   numVertices(c) nibbles before the first 0xF (the reference's
//                  numVertices table, :319-577);
//   edgeFlags(c)   derived: edge e is cut when its corners straddle the iso
//                  level (the reference's edgeFlags table, :22-55).
// Corner c of a cube at (x,y,z) is (x,y,z) + kCorner[c]
// (ReconstructionCUDA.cuh:441-452); edge e joins kEdge[e][0], kEdge[e][1].
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define FSR_HD __host__ __device__
#else
#define FSR_HD
#endif

namespace fsr {
namespace mc {

// Corner offsets and edge end points as functions (usable in device code):
// dx = bit 2, dy = bit 1, dz = bit 0 xor bit 1 reproduces kCorner below;
// edges 0-3 and 4-7 walk the x=0 and x=1 faces, edges 8-11 join them.
FSR_HD constexpr int cornerDx(int c) { return (c >> 2) & 1; }
FSR_HD constexpr int cornerDy(int c) { return (c >> 1) & 1; }
FSR_HD constexpr int cornerDz(int c) { return (c ^ (c >> 1)) & 1; }
FSR_HD constexpr int edgeA(int e) { return e < 8 ? e : e - 8; }
FSR_HD constexpr int edgeB(int e) { return e < 4 ? ((e + 1) & 3) : (e < 8 ? 4 + ((e + 1) & 3) : e - 4); }

constexpr int kCorner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0},
                               {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};

constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                              {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

constexpr uint64_t kTriPacked[256] = {
    0xffffffffffffffffULL, 0xfffffffffffff380ULL, 0xfffffffffffff910ULL, 0xffffffffff189381ULL,
    0xfffffffffffffa21ULL, 0xffffffffffa21380ULL, 0xffffffffff920a29ULL, 0xfffffff89a8a2382ULL,
    0xfffffffffffff2b3ULL, 0xffffffffff0b82b0ULL, 0xffffffffffb32091ULL, 0xfffffffb89b912b1ULL,
    0xffffffffff3ab1a3ULL, 0xfffffffab8a801a0ULL, 0xfffffff9ab9b3093ULL, 0xffffffffffb8aa89ULL,
    0xfffffffffffff874ULL, 0xffffffffff437034ULL, 0xffffffffff748910ULL, 0xfffffff137174914ULL,
    0xffffffffff748a21ULL, 0xfffffffa21403743ULL, 0xfffffff748209a29ULL, 0xffff4973727929a2ULL,
    0xffffffffff2b3748ULL, 0xfffffff40242b74bULL, 0xfffffffb32748109ULL, 0xffff1292b9b49b74ULL,
    0xfffffff487ab31a3ULL, 0xffff4b7401b41ab1ULL, 0xffff30bab9b09874ULL, 0xfffffffab99b4b74ULL,
    0xfffffffffffff459ULL, 0xffffffffff380459ULL, 0xffffffffff051450ULL, 0xfffffff513538458ULL,
    0xffffffffff459a21ULL, 0xfffffff594a21803ULL, 0xfffffff204245a25ULL, 0xffff8434535235a2ULL,
    0xffffffffffb32459ULL, 0xfffffff594b802b0ULL, 0xfffffffb32510450ULL, 0xffff584b82852512ULL,
    0xfffffff45931ab3aULL, 0xffffab81a8180594ULL, 0xffff30bab5b05045ULL, 0xfffffffb8aa85845ULL,
    0xffffffffff975879ULL, 0xfffffff375359039ULL, 0xfffffff751710870ULL, 0xffffffffff753351ULL,
    0xfffffff21a759879ULL, 0xffff37503505921aULL, 0xffff25a758528208ULL, 0xfffffff7533525a2ULL,
    0xfffffff2b3987597ULL, 0xffffb72029279759ULL, 0xffff751871810b32ULL, 0xfffffff51771b12bULL,
    0xffffb3a31a758859ULL, 0xf0aba010b7905075ULL, 0xf07570805a30b0abULL, 0xffffffffff5b75abULL,
    0xfffffffffffff56aULL, 0xffffffffff6a5380ULL, 0xffffffffff6a5109ULL, 0xfffffff6a5891381ULL,
    0xffffffffff162561ULL, 0xfffffff803621561ULL, 0xfffffff620609569ULL, 0xffff823625285895ULL,
    0xffffffffff56ab32ULL, 0xfffffff56a02b80bULL, 0xfffffff6a5b32910ULL, 0xffffb892b92916a5ULL,
    0xfffffff315356b36ULL, 0xffff6b51505b0b80ULL, 0xffff9505606306b3ULL, 0xfffffff89bb96956ULL,
    0xffffffffff8746a5ULL, 0xfffffffa56374034ULL, 0xfffffff7486a5091ULL, 0xffff49737179156aULL,
    0xfffffff874156216ULL, 0xffff743403625521ULL, 0xffff620560509748ULL, 0xf962695923497937ULL,
    0xfffffff56a4872b3ULL, 0xffffb720242746a5ULL, 0xffff6a5b32874910ULL, 0xf6a54b7b492b9129ULL,
    0xffff6b51535b3748ULL, 0xfb404b7b016b5b15ULL, 0xf74836b630560950ULL, 0xffff9b7974b96956ULL,
    0xffffffffffa4694aULL, 0xfffffff380a946a4ULL, 0xfffffff04606a10aULL, 0xffffa16468618138ULL,
    0xfffffff462421941ULL, 0xffff462942921803ULL, 0xffffffffff624420ULL, 0xfffffff624428238ULL,
    0xfffffff32b46a94aULL, 0xffff6a4a94b82280ULL, 0xffffa164606102b3ULL, 0xf1b8b12184a16146ULL,
    0xffff36b319639469ULL, 0xf14641916b0181b8ULL, 0xfffffff4600636b3ULL, 0xffffffffff86b846ULL,
    0xfffffffa98a876a7ULL, 0xffffa76a907a0370ULL, 0xffff0818717a176aULL, 0xfffffff37117a76aULL,
    0xffff768981861621ULL, 0xf937390976192962ULL, 0xfffffff206607087ULL, 0xffffffffff276237ULL,
    0xffff76898a86ab32ULL, 0xf7a9a76790b72702ULL, 0xfb32a767a1871081ULL, 0xffff17616a71b12bULL,
    0xf63136b619768698ULL, 0xffffffffff76b190ULL, 0xffff06b0b3607087ULL, 0xfffffffffffff6b7ULL,
    0xfffffffffffffb67ULL, 0xffffffffff67b803ULL, 0xffffffffff67b910ULL, 0xfffffff67b138918ULL,
    0xffffffffff7b621aULL, 0xfffffff7b6803a21ULL, 0xfffffff7b69a2092ULL, 0xffff89a38a3a27b6ULL,
    0xffffffffff726327ULL, 0xfffffff026067807ULL, 0xfffffff910732672ULL, 0xffff678891681261ULL,
    0xfffffff73171a67aULL, 0xffff801781a7167aULL, 0xffff7a69a0a70730ULL, 0xfffffff9a88a7a67ULL,
    0xffffffffff68b486ULL, 0xfffffff640603b63ULL, 0xfffffff109648b68ULL, 0xffff63b139369649ULL,
    0xfffffff1a28b6486ULL, 0xffff640b60b03a21ULL, 0xffff9a2920b648b4ULL, 0xf36463b34923a39aULL,
    0xfffffff264248328ULL, 0xffffffffff264240ULL, 0xffff834642432091ULL, 0xfffffff642241491ULL,
    0xffff1a6648168318ULL, 0xfffffff40660a01aULL, 0xf39a9303a6834364ULL, 0xffffffffff4a649aULL,
    0xffffffffffb67594ULL, 0xfffffff67b594380ULL, 0xfffffffb67045105ULL, 0xffff51345343867bULL,
    0xfffffffb6721a459ULL, 0xffff594380a217b6ULL, 0xffff204a24a45b67ULL, 0xf67b25a523453843ULL,
    0xfffffff945267327ULL, 0xffff786260680459ULL, 0xffff045051673263ULL, 0xf851584812786826ULL,
    0xffff73167161a459ULL, 0xf459078701671a61ULL, 0xfa737a6a305a4a04ULL, 0xffffa84a458a7a67ULL,
    0xfffffff98b9b6596ULL, 0xffff590650360b63ULL, 0xffffb65510b508b0ULL, 0xfffffff1355363b6ULL,
    0xffff65b8b9b59a21ULL, 0xfa21965690b603b0ULL, 0xf52025a50865b58bULL, 0xffff35a3a25363b6ULL,
    0xffff283265825985ULL, 0xfffffff260069659ULL, 0xf826283865081851ULL, 0xffffffffff612651ULL,
    0xf698965683a61631ULL, 0xffff06505960a01aULL, 0xffffffffffa65830ULL, 0xfffffffffffff65aULL,
    0xffffffffffb57a5bULL, 0xfffffff03857ba5bULL, 0xfffffff091ba57b5ULL, 0xffff1381897ba57aULL,
    0xfffffff15717b21bULL, 0xffffb27571721380ULL, 0xffff7b2209729579ULL, 0xf289823295b27257ULL,
    0xfffffff573532a52ULL, 0xffff52a578258028ULL, 0xffff2a37353a5109ULL, 0xf25752a278129289ULL,
    0xffffffffff573531ULL, 0xfffffff571170780ULL, 0xfffffff735539309ULL, 0xffffffffff795789ULL,
    0xfffffff8ba8a5485ULL, 0xffff03bba50b5405ULL, 0xffff54aba8a48910ULL, 0xf41314943b54a4baULL,
    0xffff8548b2582152ULL, 0xfb151b2b543b0b40ULL, 0xf58b8545b2950520ULL, 0xffffffffff3b2549ULL,
    0xffff483543253a52ULL, 0xfffffff0244252a5ULL, 0xf910854583a532a3ULL, 0xffff2492914252a5ULL,
    0xfffffff153358548ULL, 0xffffffffff501540ULL, 0xffff530509358548ULL, 0xfffffffffffff549ULL,
    0xfffffffba9b947b4ULL, 0xffffba97b9794380ULL, 0xffffb470414b1ba1ULL, 0xf4bab474a1843413ULL,
    0xffff219b294b97b4ULL, 0xf3801b2b197b9479ULL, 0xfffffff04224b47bULL, 0xffff42343824b47bULL,
    0xffff947732972a92ULL, 0xf70207872a4797a9ULL, 0xfa040a1a472a3a73ULL, 0xffffffffff4782a1ULL,
    0xfffffff317714194ULL, 0xffff178180714194ULL, 0xffffffffff347304ULL, 0xfffffffffffff784ULL,
    0xffffffffff8ba8a9ULL, 0xfffffffa9bb93903ULL, 0xfffffffba88a0a10ULL, 0xffffffffffa3ba13ULL,
    0xfffffff8b99b1b21ULL, 0xffff9b2921b93903ULL, 0xffffffffffb08b20ULL, 0xfffffffffffffb23ULL,
    0xfffffff98aa82832ULL, 0xffffffffff2902a9ULL, 0xffff8a1810a82832ULL, 0xfffffffffffff2a1ULL,
    0xffffffffff819831ULL, 0xfffffffffffff190ULL, 0xfffffffffffff830ULL, 0xffffffffffffffffULL,
};

constexpr unsigned numVertices(unsigned c)
{
    unsigned k = 0;
    while (k < 16u && ((kTriPacked[c] >> (4u * k)) & 0xFu) != 0xFu) ++k;
    return k;
}

constexpr unsigned edgeFlags(unsigned c)
{
    unsigned m = 0;
    for (unsigned e = 0; e < 12u; ++e)
        if (((c >> kEdge[e][0]) & 1u) != ((c >> kEdge[e][1]) & 1u)) m |= 1u << e;
    return m;
}

struct Derived {
    uint8_t nverts[256];
    uint16_t eflags[256];
};

constexpr Derived derive()
{
    Derived d{};
    for (unsigned c = 0; c < 256; ++c) {
        d.nverts[c] = (uint8_t)numVertices(c);
        d.eflags[c] = (uint16_t)edgeFlags(c);
    }
    return d;
}

constexpr Derived kDerived = derive();

constexpr bool checkFunctions()
{
    for (int c = 0; c < 8; ++c)
        if (cornerDx(c) != kCorner[c][0] || cornerDy(c) != kCorner[c][1] || cornerDz(c) != kCorner[c][2])
            return false;
    for (int e = 0; e < 12; ++e)
        if (edgeA(e) != kEdge[e][0] || edgeB(e) != kEdge[e][1]) return false;
    return true;
}
static_assert(checkFunctions(), "corner/edge functions match the tables");
static_assert(numVertices(0) == 0 && numVertices(255) == 0, "empty cases");
static_assert(edgeFlags(1) == 0x109, "corner 0 cuts edges 0, 3 and 8");

}  // namespace mc
}  // namespace fsr
