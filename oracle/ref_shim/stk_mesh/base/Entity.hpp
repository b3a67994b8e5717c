#pragma once
namespace stk { namespace mesh { struct Entity { unsigned long m_value = 0; }; } }
