// Headless Image for the reference's Renderer (Core/include/Image.h:13-27
// declares it over Vulkan; Renderer.cu creates one per resize and hands it the
// RGBA8 pixels each frame).  Same constructor and the members Renderer.cu
// calls; setData keeps a host copy of the pixels instead of uploading them.
#pragma once

#include <cstdint>
#include <cstring>
#include <string_view>
#include <vector>

enum class ImageType
{
    None = 0,
    RGBA,
    RGBA32F
};

class Image
{
public:
    Image(uint32_t width, uint32_t height, ImageType type, const void* data = nullptr)
        : m_width(width), m_height(height), m_type(type),
          m_pixels(static_cast<size_t>(width) * height * (type == ImageType::RGBA32F ? 16 : 4))
    {
        if (data) setData(data);
    }

    void setData(const void* data) { std::memcpy(m_pixels.data(), data, m_pixels.size()); }
    const void* pixels() const { return m_pixels.data(); }

    uint32_t getWidth() const { return m_width; }
    uint32_t getHeight() const { return m_height; }

private:
    uint32_t m_width = 0, m_height = 0;
    ImageType m_type = ImageType::None;
    std::vector<unsigned char> m_pixels;
};
