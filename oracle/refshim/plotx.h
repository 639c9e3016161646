/*
 * plotx.h -- stand-in for the PlotX plotting library so that the reference's
 * src/singlepulse/candidate.cpp compiles in place; every call is accepted and draws nothing.
 * Test infrastructure only.
 */
#ifndef TXREF_PLOTX_H
#define TXREF_PLOTX_H
#include <map>
#include <string>
namespace PlotX {
using Opts = std::map<std::string, std::string>;
#define TXREF_ANY(name)                                                                           \
    template <class... A> void name(A &&...) {}                                                 \
    template <class A1> void name(A1 &&, Opts) {}                                               \
    template <class A1, class A2> void name(A1 &&, A2 &&, Opts) {}                              \
    template <class A1, class A2, class A3> void name(A1 &&, A2 &&, A3 &&, Opts) {}             \
    template <class A1, class A2, class A3, class A4> void name(A1 &&, A2 &&, A3 &&, A4 &&, Opts) {} \
    template <class A1, class A2, class A3, class A4, class A5>                                 \
    void name(A1 &&, A2 &&, A3 &&, A4 &&, A5 &&, Opts) {}
struct Axes {
    template <class... A> Axes(A &&...) {}
    TXREF_ANY(annotate) TXREF_ANY(axhline) TXREF_ANY(axvline) TXREF_ANY(set_ylabel)
    TXREF_ANY(set_xlabel) TXREF_ANY(pcolor) TXREF_ANY(label) TXREF_ANY(plot) TXREF_ANY(autoscale)
    TXREF_ANY(minorticks_off) TXREF_ANY(majorticks_off) TXREF_ANY(frame) TXREF_ANY(circle)
    TXREF_ANY(set_xlim) TXREF_ANY(set_ylim) TXREF_ANY(errorbar) TXREF_ANY(scatter)
    TXREF_ANY(legend) TXREF_ANY(text) TXREF_ANY(colorbar) TXREF_ANY(set_title)
};
struct Figure {
    template <class... A> Figure(A &&...) {}
    TXREF_ANY(push) TXREF_ANY(set_default_color) TXREF_ANY(set_background_color) TXREF_ANY(show)
    TXREF_ANY(save) TXREF_ANY(savepx) TXREF_ANY(close)
#undef TXREF_ANY
};
#undef TXREF_ANY
} // namespace PlotX
#endif
