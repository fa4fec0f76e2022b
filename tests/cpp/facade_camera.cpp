// Drives axr::Camera (include/axr.hpp) with a camera script and writes the matrices and
// position after every operation: the C++ facade's camera against the reference's.
// usage: facade_camera script.bin out.bin
//   script: 8 floats (position, target, fov, aspect), u32 n, then n ops of 6 floats
//   (kind, a0..a3, flags; tests/camscript.py); out: n x 51 floats.
#include <cstdio>
#include <vector>

#include "axr.hpp"

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    float start[8];
    uint32_t n = 0;
    if (std::fread(start, 4, 8, f) != 8 || std::fread(&n, 4, 1, f) != 1) return 2;
    std::vector<float> ops(6ull * n);
    if (std::fread(ops.data(), 4, ops.size(), f) != ops.size()) return 2;
    std::fclose(f);
    // the bare constructor state: the script starts before any update
    axr_camera_state st{};
    axr::check(axr_camera_init(&st, start, start + 3, start[6], start[7]));
    axr::check(axr_camera_set_viewport(&st, 0, 0, 800, 600));
    std::vector<float> out(51ull * n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* o = &ops[6ull * i];
        switch (int(o[0])) {
            case 0: axr::check(axr_camera_update(&st, o[1])); break;
            case 1: {
                axr_input_state in{};
                in.mouse[0] = o[1];
                in.mouse[1] = o[2];
                const int flags = int(o[5]);
                in.mouse_buttons[1] = (flags & 1) ? 1 : 0;
                const char keys[4] = {'W', 'S', 'A', 'D'};
                for (int k = 0; k < 4; ++k) in.keys[(unsigned char)keys[k]] = (flags & (2 << k)) ? 1 : 0;
                axr::check(axr_camera_handle_input(&st, &in));
                break;
            }
            case 2: axr::check(axr_camera_set_position(&st, o + 1)); break;
            case 3: axr::check(axr_camera_set_target(&st, o + 1)); break;
            case 4: axr::check(axr_camera_set_fov(&st, o[1])); break;
            case 5: axr::check(axr_camera_set_aspect_ratio(&st, o[1])); break;
            case 6: axr::check(axr_camera_set_viewport(&st, int(o[1]), int(o[2]), int(o[3]), int(o[4]))); break;
            default: return 3;
        }
        float* r = &out[51ull * i];
        std::copy(st.view, st.view + 16, r);
        std::copy(st.projection, st.projection + 16, r + 16);
        std::copy(st.view_proj, st.view_proj + 16, r + 32);
        std::copy(st.position, st.position + 3, r + 48);
    }
    // the facade class: constructor + update(0), then a drag and a move
    axr::Camera cam({start[0], start[1], start[2]}, {start[3], start[4], start[5]}, start[6], start[7]);
    axr::InputState in;
    in.mouseX = 10;
    in.mouseY = 10;
    in.rightButton = true;
    cam.handleInput(in);
    in.mouseX = 40;
    in.mouseY = 25;
    in.keys['W'] = true;
    cam.handleInput(in);
    cam.update(0.1f);
    const axr::Mat4 vp = cam.getViewProjectionMatrix();
    out.insert(out.end(), vp.begin(), vp.end());
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(out.data(), 4, out.size(), f);
    std::fclose(f);
    return 0;
}
