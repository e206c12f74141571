// Headless input for the reference's Camera.cpp (Camera::onUpdate polls
// Input::Input, Core/include/input/Input.h:8-18, which the reference backs
// with GLFW in Core/src/input/Input.cpp).  Same class and static functions;
// they read a state the caller sets (ref_input_state()), so a test can drive
// the reference's camera motion with chosen keys, button and mouse position.
// The key, button and cursor-mode enums are the reference's own KeyCodes.h.
#pragma once

#include "input/KeyCodes.h"

#include <glm/glm.hpp>

namespace Input
{
struct RefInputState
{
    bool keys[512];
    bool right_button;
    float mouse_x, mouse_y;
    int cursor_mode;
};

inline RefInputState& ref_input_state()
{
    static RefInputState s{};
    return s;
}

class Input
{
public:
    static bool IsKeyPressed(KeyCode key)
    {
        const unsigned k = static_cast<unsigned>(key);
        return k < 512 && ref_input_state().keys[k];
    }
    static bool IsMouseButtonPressed(MouseButton button)
    {
        return button == MouseButton::Right && ref_input_state().right_button;
    }
    static glm::vec2 GetMousePosition() { return {ref_input_state().mouse_x, ref_input_state().mouse_y}; }
    static void SetCursorMode(CursorMode mode) { ref_input_state().cursor_mode = static_cast<int>(mode); }
};
}  // namespace Input
