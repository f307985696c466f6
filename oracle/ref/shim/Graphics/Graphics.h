// Stand-in for the engine's Graphics/Graphics.h (Vulkan/evk), providing only
// what Sources/World/Systems/ShadowVoxSystem.cpp touches: a host byte buffer,
// an image extent, and a synchronous "transfer" that records copy regions.
// Part of the oracle's reference-build recipe (test infrastructure).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

typedef uint8_t uint8;
typedef uint32_t uint32;
typedef uint64_t uint64;
typedef int32_t int32;

enum class Format { R8Uint };
enum class ImageLayout { Undefined, TransferDst, ShaderReadOptimal };
struct Extent {
    uint32_t width, height, depth;
};
struct ImageRegion {
    int x, y, z;
    uint32_t width, height, depth, mip{0}, layer{0};
};
struct Image {
    Extent ext{0, 0, 0};
    struct Info {
        Format format;
        Extent extent;
        Info(Format f, Extent e) : format(f), extent(e) {}
    };
    static Image Create(const Info& i) {
        Image im;
        im.ext = i.extent;
        return im;
    }
    Extent getExtent() { return ext; }
};
struct Buffer {
    std::shared_ptr<std::vector<uint8_t>> mem;
    static Buffer Create(uint64_t size);
    void* getData() { return mem ? mem->data() : nullptr; }
};
// the most recently created buffer and the regions of the most recent copy
struct ShimTransferLog {
    std::shared_ptr<std::vector<uint8_t>> last_buffer;
    std::vector<ImageRegion> regions;
    int copies = 0;
};
inline ShimTransferLog& shim_log() {
    static ShimTransferLog l;
    return l;
}
inline Buffer Buffer::Create(uint64_t size) {
    Buffer b;
    b.mem = std::make_shared<std::vector<uint8_t>>(size, 0xAB);  // garbage until the ctor clears it
    shim_log().last_buffer = b.mem;
    return b;
}
struct CmdBuffer {
    void barrier(Image&, ImageLayout, ImageLayout) {}
    void copy(Buffer&, Image&, const std::vector<ImageRegion>& r) {
        shim_log().regions.insert(shim_log().regions.end(), r.begin(), r.end());
        shim_log().copies++;
    }
};
class Graphics {
public:
    template <typename T>
    static void Transfer(T callback) {
        CmdBuffer c;
        callback(c);
    }
};
