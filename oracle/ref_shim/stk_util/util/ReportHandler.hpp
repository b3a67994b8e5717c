#pragma once
#include <stdexcept>
#include <string>
#define STK_ThrowAssert(x) ((void)0)
#define STK_ThrowAssertMsg(x, m) ((void)0)
#define STK_ThrowRequire(x) do { if (!(x)) throw std::runtime_error(#x); } while (0)
#define STK_ThrowRequireMsg(x, m) do { if (!(x)) throw std::runtime_error(#x); } while (0)
#define STK_ThrowErrorMsg(m) throw std::runtime_error("stk error")
