// Stand-in for Cem Yuksel's cyHairFile (an absent submodule of the
// reference; cyCodeBase), for the host build of the reference's scene.cpp.
// Test infrastructure only.  It keeps the names scene.cpp uses and reads
// the published HAIR format: a 128-byte header ("HAIR", hair count, point
// count, array bits: 1 segments, 2 points, 4 thickness, 8 transparency,
// 16 colors; default segments, thickness, transparency, color[3], 88 bytes
// of information), then the arrays present in that order: segments
// (uint16 per strand), points (3 x float32 per point), thickness (float32),
// transparency (float32), colors (3 x float32).
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#define CY_HAIR_FILE_SEGMENTS_BIT 1
#define CY_HAIR_FILE_POINTS_BIT 2
#define CY_HAIR_FILE_THICKNESS_BIT 4
#define CY_HAIR_FILE_TRANSPARENCY_BIT 8
#define CY_HAIR_FILE_COLORS_BIT 16

#define CY_HAIR_FILE_ERROR_CANT_OPEN_FILE -1
#define CY_HAIR_FILE_ERROR_CANT_READ_HEADER -2
#define CY_HAIR_FILE_ERROR_WRONG_SIGNATURE -3
#define CY_HAIR_FILE_ERROR_READING_SEGMENTS -4
#define CY_HAIR_FILE_ERROR_READING_POINTS -5
#define CY_HAIR_FILE_ERROR_READING_COLORS -6
#define CY_HAIR_FILE_ERROR_READING_THICKNESS -7
#define CY_HAIR_FILE_ERROR_READING_TRANSPARENCY -8

class cyHairFile {
 public:
  struct Header {
    char signature[4];
    unsigned int hair_count;
    unsigned int point_count;
    unsigned int arrays;
    unsigned int d_segments;
    float d_thickness;
    float d_transparency;
    float d_color[3];
    char info[88];
  };
  cyHairFile() { memset(&header, 0, sizeof(header)); }
  const Header& GetHeader() const { return header; }
  const unsigned short* GetSegmentsArray() const { return segments.empty() ? nullptr : segments.data(); }
  const float* GetPointsArray() const { return points.empty() ? nullptr : points.data(); }
  const float* GetThicknessArray() const { return thickness.empty() ? nullptr : thickness.data(); }
  int LoadFromFile(const char* filename) {
    FILE* f = fopen(filename, "rb");
    if (!f) return CY_HAIR_FILE_ERROR_CANT_OPEN_FILE;
    static_assert(sizeof(Header) == 128, "HAIR header is 128 bytes");
    if (fread(&header, sizeof(Header), 1, f) < 1) return fclose(f), CY_HAIR_FILE_ERROR_CANT_READ_HEADER;
    if (strncmp(header.signature, "HAIR", 4) != 0) return fclose(f), CY_HAIR_FILE_ERROR_WRONG_SIGNATURE;
    segments.clear(); points.clear(); thickness.clear();
    if (header.arrays & CY_HAIR_FILE_SEGMENTS_BIT) {
      segments.resize(header.hair_count);
      if (fread(segments.data(), 2, header.hair_count, f) < header.hair_count)
        return fclose(f), CY_HAIR_FILE_ERROR_READING_SEGMENTS;
    }
    if (header.arrays & CY_HAIR_FILE_POINTS_BIT) {
      points.resize((size_t)header.point_count * 3);
      if (fread(points.data(), 4, points.size(), f) < points.size()) return fclose(f), CY_HAIR_FILE_ERROR_READING_POINTS;
    }
    if (header.arrays & CY_HAIR_FILE_THICKNESS_BIT) {
      thickness.resize(header.point_count);
      if (fread(thickness.data(), 4, thickness.size(), f) < thickness.size())
        return fclose(f), CY_HAIR_FILE_ERROR_READING_THICKNESS;
    }
    fclose(f);
    return (int)header.hair_count;
  }

 private:
  Header header;
  std::vector<unsigned short> segments;
  std::vector<float> points, thickness;
};
