/* Headless replacement for FVMR/src/gui/WinGui.h (declared at lines 13-21
 * there).  The oracle build never opens a window; FVMR/src/drivers/CDriver.h
 * only needs the class and the members it names.  The symlink farm points
 * gui/WinGui.h at this file.  Oracle build only. */
#pragma once
class WinGui {
public:
	void init() {}
	void render() {}
	void cleanup() {}
	bool windowShouldClose() { return false; }
	void set_enabled(bool b) { m_enabled = b; }
	bool get_enabled() { return m_enabled; }
	bool& get_enabled_ref() { return m_enabled; }
private:
	bool m_enabled = false;
};
