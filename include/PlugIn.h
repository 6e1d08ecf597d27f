/* PlugIn.h - headless plugin interface and frame loop (PlugIn.h:88-92 of the
 * reference, without the GLUT demo).
 *
 * A plugin keeps the reference's life cycle: open(), then update(t, dt)
 * every frame, redraw(t, dt) when a frame is to be shown, close(); reset()
 * is close() + open().  redraw() is where a plugin reads its agents back to
 * the host (SyncHost / GetDataForAgent); with no graphics stack there is no
 * drawing.  Plugins register themselves by construction, as in the
 * reference, and runHeadless() replaces the demo's main loop. */
#ifndef GPUSTEER_PLUGIN_H
#define GPUSTEER_PLUGIN_H

#include <algorithm>
#include <cstring>
#include <vector>

namespace OpenSteer {

class AbstractPlugIn {
public:
    virtual ~AbstractPlugIn() {}
    virtual void open() = 0;
    virtual void update(const float currentTime, const float elapsedTime) = 0;
    virtual void redraw(const float currentTime, const float elapsedTime) = 0;
    virtual void close() = 0;
    virtual void reset() = 0;
    virtual const char* name() = 0;
    virtual float selectionOrderSortKey() = 0;
    virtual bool requestInitialSelection() = 0;
};

class PlugIn : public AbstractPlugIn {
public:
    PlugIn() { registry().push_back(this); }
    virtual ~PlugIn() {
        auto& r = registry();
        r.erase(std::remove(r.begin(), r.end(), this), r.end());
    }
    void reset() { close(); open(); }
    float selectionOrderSortKey() { return 1.0f; }
    bool requestInitialSelection() { return false; }

    static PlugIn* findByName(const char* string) {
        for (PlugIn* p : registry())
            if (std::strcmp(p->name(), string) == 0) return p;
        return nullptr;
    }
    static std::vector<PlugIn*>& registry() {
        static std::vector<PlugIn*> r;
        return r;
    }
};

/* The frame loop without a window: open, `frames` updates of elapsedTime
 * (redraw every `redrawEvery` frames when non-zero), close. */
inline void runHeadless(AbstractPlugIn& plugin, unsigned frames, float elapsedTime,
                        unsigned redrawEvery = 0) {
    plugin.open();
    float t = 0.f;
    for (unsigned f = 0; f < frames; ++f) {
        t += elapsedTime;
        plugin.update(t, elapsedTime);
        if (redrawEvery && (f + 1) % redrawEvery == 0) plugin.redraw(t, elapsedTime);
    }
    plugin.close();
}

}  // namespace OpenSteer

#endif
