// tensor_flag / tensor_flags as in the reference (src/tensor.h:12-62), for
// the template signatures of the shims.
#pragma once

namespace fdm {

enum struct tensor_flag : int { none = 0, periodic = 1 };

template <tensor_flag... Args>
struct tensor_flags;

template <tensor_flag Head, tensor_flag... Tail>
struct tensor_flags<Head, Tail...> {
    using tail = tensor_flags<Tail...>;
    static constexpr tensor_flag head = Head;
};

template <>
struct tensor_flags<> {
    using tail = tensor_flags<>;
    static constexpr tensor_flag head = tensor_flag::none;
};

// bit mask of periodic axes for the C ABI (bit 0 = x, 1 = y, 2 = z; the
// reference lists flags z, y, x)
template <typename F>
struct tensor_flags_mask {
    static constexpr int value = (F::head == tensor_flag::periodic ? 4 : 0) |
                                 (F::tail::head == tensor_flag::periodic ? 2 : 0) |
                                 (F::tail::tail::head == tensor_flag::periodic ? 1 : 0);
};

}  // namespace fdm
