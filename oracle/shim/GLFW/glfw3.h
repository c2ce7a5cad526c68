// Type-only stand-in for GLFW (test infrastructure; nothing is called).
#pragma once
struct GLFWwindow;
