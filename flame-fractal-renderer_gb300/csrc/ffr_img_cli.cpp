// ffr-img: buffer -> PNG front end over libffr_gpu.so's C ABI.
//
// Same options, checks and stderr report as the reference's
// src/ffr_img.cpp:61-197 (-f/--flame, -i/--input (repeatable, '-' =
// stdin), -o/--output ('-' = stdout), -y/--gamma (default 1), -m/--monochrome,
// -g/--grayscale, -c/--color, -b/--bits 8|16); the buffers are added and
// mapped to pixels on the device (ffr_render_image) and the PNG is encoded
// on the host (ffr_encode_png).  Errors that the reference throws out of
// main print "ERROR: <message>" and exit 1 here.
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include "ffr_gpu.h"

namespace {

const char* kUsage =
    "ffr-img usage:\n"
    "  -h [ --help ]             show this help message\n"
    "  -f [ --flame ] arg        flame parameters JSON file\n"
    "  -i [ --input ] arg        buffers to add\n"
    "  -o [ --output ] arg       output file\n"
    "  -y [ --gamma ] arg (=1)   gamma value\n"
    "  -m [ --monochrome ]       binary image from histogram\n"
    "  -g [ --grayscale ]        grayscale image from histogram\n"
    "  -c [ --color ]            color image from 3d color only\n"
    "  -b [ --bits ] arg (=8)    bits per color channel\n"
    "  --device arg (=0)         CUDA device\n";

[[noreturn]] void die(const std::string& m)
{
    std::cerr << "ERROR: " << m << std::endl;
    std::exit(1);
}

std::string read_all(std::istream& in)
{
    return std::string((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

void check(ffr_ctx* ctx, ffr_status s)
{
    if (s != FFR_OK)
        die(ffr_last_error(ctx));
}

} // namespace

int main(int argc, char** argv)
{
    std::string flame, output;
    std::vector<std::string> inputs;
    double gamma = 1.0;
    uint64_t bits = 8;
    int device = 0;
    bool m = false, g = false, c = false, help = false, have_flame = false, have_output = false;
    for (int k = 1; k < argc; ++k)
    {
        std::string t = argv[k];
        auto value = [&](const std::string& name) -> std::string {
            if (k + 1 >= argc)
                die("the required argument for option '--" + name + "' is missing");
            return argv[++k];
        };
        if (t == "-h" || t == "--help") help = true;
        else if (t == "-f" || t == "--flame") { flame = value("flame"); have_flame = true; }
        else if (t == "-i" || t == "--input") inputs.push_back(value("input"));
        else if (t == "-o" || t == "--output") { output = value("output"); have_output = true; }
        else if (t == "-y" || t == "--gamma")
        {
            const std::string v = value("gamma");
            char* end = nullptr;
            errno = 0;
            gamma = std::strtod(v.c_str(), &end);
            if (errno || *end || v.empty())
                die("the argument ('" + v + "') for option '--gamma' is invalid");
        }
        else if (t == "-m" || t == "--monochrome") m = true;
        else if (t == "-g" || t == "--grayscale") g = true;
        else if (t == "-c" || t == "--color") c = true;
        else if (t == "-b" || t == "--bits")
        {
            const std::string v = value("bits");
            char* end = nullptr;
            bits = std::strtoull(v.c_str(), &end, 10);
            if (*end || v.empty() || v[0] == '-')
                die("the argument ('" + v + "') for option '--bits' is invalid");
        }
        else if (t == "--device") device = std::atoi(value("device").c_str());
        else
            die("unrecognised option '" + t + "'");
    }
    if (help || argc < 2)
    {
        std::cerr << kUsage;
        return 1;
    }
    if (!have_flame)
        die("the option '--flame' is required but missing");
    if (!have_output)
        die("the option '--output' is required but missing");
    // ffr_img.cpp:89-95
    if (gamma < 1e-20)
        die("gamma too small");
    if (bits != 8 && bits != 16)
        die("bits per channel must be 8 or 16");

    // option echo (ffr_img.cpp:97-113)
    std::cerr << "ffr-img version gb300" << std::endl;
    std::cerr << "--flame " << flame << std::endl;
    for (auto& s : inputs)
        std::cerr << "--input " << s << std::endl;
    std::cerr << "--output " << output << std::endl;
    std::cerr << "--gamma " << gamma << std::endl;
    if (m)
        std::cerr << "--monochrome" << std::endl;
    if (g)
        std::cerr << "--grayscale" << std::endl;
    if (c)
        std::cerr << "--color" << std::endl;
    std::cerr << "--bits " << bits << std::endl;
    std::cerr << "--" << std::endl;

    std::string text;
    if (flame == "-")
        text = read_all(std::cin);
    else
    {
        std::ifstream f(flame, std::ios::in | std::ios::binary);
        if (!f)
            die("cannot open flame file " + flame);
        text = read_all(f);
    }
    ffr_opts o;
    ffr_default_opts(&o);
    o.device = device;
    ffr_ctx* ctx = nullptr;
    if (ffr_create(text.data(), text.size(), &o, &ctx) != FFR_OK)
        die(ffr_last_error(nullptr));
    std::cerr << "flame: " << ffr_flame_json(ctx) << std::endl;
    uint32_t dims = 0, color_dims = 0;
    uint64_t cells = 0;
    size_t bytes = 0;
    check(ctx, ffr_info(ctx, &dims, &cells, &color_dims, &bytes));
    if (dims != 2)
    {
        std::cerr << "ERROR: only 2D flames supported" << std::endl;
        return 1;
    }
    std::cerr << "buffer: " << bytes << " bytes, little endian, 8 byte numbers" << std::endl;
    std::cerr << "color: " << color_dims << " dimensions" << std::endl;
    if ((int)m + (int)g + (int)c != 1)
    {
        std::cerr << "ERROR: must choose exactly 1 coloring flag "
                  << "(--monochrome, --grayscale, --color)" << std::endl;
        return 1;
    }
    if (inputs.empty())
    {
        std::cerr << "ERROR: no input buffer files specified" << std::endl;
        return 1;
    }
    std::vector<char> buf(bytes);
    for (auto& s : inputs)
    {
        std::cerr << "adding input file " << s << std::endl;
        bool ok;
        if (s == "-")
        {
            std::cin.read(buf.data(), (std::streamsize)buf.size());
            ok = (size_t)std::cin.gcount() == buf.size();
        }
        else
        {
            std::ifstream f(s, std::ios::in | std::ios::binary);
            f.read(buf.data(), (std::streamsize)buf.size());
            ok = f && (size_t)f.gcount() == buf.size();
        }
        if (!ok)
            die("error reading file");
        check(ctx, ffr_add_buffer(ctx, buf.data(), buf.size()));
    }

    std::cerr << "processing buffer" << std::endl;
    const int mode = m ? FFR_IMAGE_MONO : (g ? FFR_IMAGE_GRAY : FFR_IMAGE_RGB);
    const uint32_t ch = mode == FFR_IMAGE_RGB ? 3 : 1;
    const uint32_t pbits = mode == FFR_IMAGE_MONO ? 8 : (uint32_t)bits;
    std::vector<unsigned char> pixels((size_t)cells * ch * (pbits / 8));
    ffr_image_info info{};
    ffr_status st = ffr_render_image(ctx, mode, gamma, (uint32_t)bits, pixels.data(),
                                     pixels.size(), &info);
    if (st == FFR_OK || st == FFR_ERR_STATE)
    {
        std::cerr << "histogram bounds: " << info.hist_min << " " << info.hist_max << std::endl;
        std::cerr << "scaler bounds: " << info.scale_min << " " << info.scale_max << std::endl;
    }
    check(ctx, st);
    size_t len = 0;
    ffr_encode_png(pixels.data(), info.width, info.height, ch, pbits, nullptr, 0, &len);
    std::vector<unsigned char> png(len);
    if (ffr_encode_png(pixels.data(), info.width, info.height, ch, pbits, png.data(), png.size(),
                       &len) != FFR_OK)
        die("error writing output");
    bool ok;
    if (output == "-")
    {
        std::cout.write(reinterpret_cast<const char*>(png.data()), (std::streamsize)png.size());
        std::cout.flush();
        ok = std::cout.good();
    }
    else
    {
        std::ofstream f(output, std::ios::out | std::ios::binary);
        f.write(reinterpret_cast<const char*>(png.data()), (std::streamsize)png.size());
        ok = f.good();
    }
    if (!ok)
        die("error writing output");
    ffr_destroy(ctx);
    return 0;
}
