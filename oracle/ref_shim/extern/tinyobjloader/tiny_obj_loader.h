// Compile-only stand-in for tinyobjloader used when compiling the reference sources.
// TEST INFRASTRUCTURE ONLY: mesh scenes are not part of the denoise path, so
// ParseFromFile always fails and the mesh lists stay empty.
#pragma once
#include <string>
#include <vector>
namespace tinyobj {
struct ObjReaderConfig {};
struct index_t { int vertex_index = 0; int normal_index = 0; int texcoord_index = 0; };
struct mesh_t { std::vector<index_t> indices; std::vector<unsigned char> num_face_vertices; };
struct shape_t { std::string name; mesh_t mesh; };
struct attrib_t { std::vector<float> vertices; };
class ObjReader {
public:
    bool ParseFromFile(const std::string&, const ObjReaderConfig& = ObjReaderConfig()) { return false; }
    const std::string& Error() const { return err_; }
    const std::string& Warning() const { return warn_; }
    const attrib_t& GetAttrib() const { return attrib_; }
    const std::vector<shape_t>& GetShapes() const { return shapes_; }
private:
    std::string err_ = "mesh loading is not available in the oracle harness";
    std::string warn_;
    attrib_t attrib_;
    std::vector<shape_t> shapes_;
};
}  // namespace tinyobj
