// operator_cuda.cpp -- Operator_CUDA (see operator_cuda.h).
#include "operator_cuda.h"

#include <iostream>

#include "engine_cuda.h"
#include "FDTD/extensions/operator_ext_excitation.h"
#include "FDTD/extensions/operator_ext_lorentzmaterial.h"
#include "FDTD/extensions/operator_ext_lumpedRLC.h"
#include "FDTD/extensions/operator_ext_mur_abc.h"
#include "FDTD/extensions/operator_ext_upml.h"

namespace {

// The extensions keep their arrays protected (their own engine extensions
// are their friends).  A pointer to a protected member, formed inside a
// class derived from the extension, may be applied to any object of the
// extension's class: the glue reads the arrays through such pointers and
// the reference's headers need no change.
struct UpmlAccess : Operator_Ext_UPML
{
	typedef FDTD_FLOAT**** Operator_Ext_UPML::*Arr;
	static Arr vv_() {return &UpmlAccess::vv;}
	static Arr vvfo_() {return &UpmlAccess::vvfo;}
	static Arr vvfn_() {return &UpmlAccess::vvfn;}
	static Arr ii_() {return &UpmlAccess::ii;}
	static Arr iifo_() {return &UpmlAccess::iifo;}
	static Arr iifn_() {return &UpmlAccess::iifn;}
	static unsigned int (Operator_Ext_UPML::*start_())[3] {return &UpmlAccess::m_StartPos;}
	static unsigned int (Operator_Ext_UPML::*lines_())[3] {return &UpmlAccess::m_numLines;}
};

struct LorentzAccess : Operator_Ext_LorentzMaterial
{
	typedef FDTD_FLOAT*** Operator_Ext_LorentzMaterial::*Arr;
	static Arr v_int_() {return &LorentzAccess::v_int_ADE;}
	static Arr v_ext_() {return &LorentzAccess::v_ext_ADE;}
	static Arr v_lor_() {return &LorentzAccess::v_Lor_ADE;}
	static Arr i_int_() {return &LorentzAccess::i_int_ADE;}
	static Arr i_ext_() {return &LorentzAccess::i_ext_ADE;}
	static Arr i_lor_() {return &LorentzAccess::i_Lor_ADE;}
	static bool* Operator_Ext_LorentzMaterial::*volt_lor_on_() {return &LorentzAccess::m_volt_Lor_ADE_On;}
	static bool* Operator_Ext_LorentzMaterial::*curr_lor_on_() {return &LorentzAccess::m_curr_Lor_ADE_On;}
	static int Operator_Ext_Dispersive::*order_() {return &LorentzAccess::m_Order;}
	static std::vector<unsigned int> Operator_Ext_Dispersive::*count_() {return &LorentzAccess::m_LM_Count;}
	static unsigned int*** Operator_Ext_Dispersive::*pos_() {return &LorentzAccess::m_LM_pos;}
	static bool* Operator_Ext_Dispersive::*volt_on_() {return &LorentzAccess::m_volt_ADE_On;}
	static bool* Operator_Ext_Dispersive::*curr_on_() {return &LorentzAccess::m_curr_ADE_On;}
};

struct ExcitationAccess : Operator_Ext_Excitation
{
	static unsigned int Operator_Ext_Excitation::*volt_count_() {return &ExcitationAccess::Volt_Count;}
	static unsigned int* (Operator_Ext_Excitation::*volt_index_())[3] {return &ExcitationAccess::Volt_index;}
	static unsigned short* Operator_Ext_Excitation::*volt_dir_() {return &ExcitationAccess::Volt_dir;}
	static FDTD_FLOAT* Operator_Ext_Excitation::*volt_amp_() {return &ExcitationAccess::Volt_amp;}
	static unsigned int* Operator_Ext_Excitation::*volt_delay_() {return &ExcitationAccess::Volt_delay;}
	static unsigned int Operator_Ext_Excitation::*curr_count_() {return &ExcitationAccess::Curr_Count;}
	static unsigned int* (Operator_Ext_Excitation::*curr_index_())[3] {return &ExcitationAccess::Curr_index;}
	static unsigned short* Operator_Ext_Excitation::*curr_dir_() {return &ExcitationAccess::Curr_dir;}
	static FDTD_FLOAT* Operator_Ext_Excitation::*curr_amp_() {return &ExcitationAccess::Curr_amp;}
	static unsigned int* Operator_Ext_Excitation::*curr_delay_() {return &ExcitationAccess::Curr_delay;}
};

struct MurAccess : Operator_Ext_Mur_ABC
{
	static int Operator_Ext_Mur_ABC::*ny_() {return &MurAccess::m_ny;}
	static int Operator_Ext_Mur_ABC::*nyP_() {return &MurAccess::m_nyP;}
	static int Operator_Ext_Mur_ABC::*nyPP_() {return &MurAccess::m_nyPP;}
	static bool Operator_Ext_Mur_ABC::*top_() {return &MurAccess::m_top;}
	static unsigned int Operator_Ext_Mur_ABC::*line_() {return &MurAccess::m_LineNr;}
	static int Operator_Ext_Mur_ABC::*shift_() {return &MurAccess::m_LineNr_Shift;}
	static unsigned int (Operator_Ext_Mur_ABC::*lines_())[2] {return &MurAccess::m_numLines;}
	static FDTD_FLOAT** Operator_Ext_Mur_ABC::*coef_p_() {return &MurAccess::m_Mur_Coeff_nyP;}
	static FDTD_FLOAT** Operator_Ext_Mur_ABC::*coef_pp_() {return &MurAccess::m_Mur_Coeff_nyPP;}
};

struct RlcAccess : Operator_Ext_LumpedRLC
{
	typedef FDTD_FLOAT* Operator_Ext_LumpedRLC::*Arr;
	static unsigned int Operator_Ext_LumpedRLC::*count_() {return &RlcAccess::RLC_count;}
	static unsigned int** Operator_Ext_LumpedRLC::*pos_() {return &RlcAccess::v_RLC_pos;}
	static int* Operator_Ext_LumpedRLC::*dir_() {return &RlcAccess::v_RLC_dir;}
	static void coefs(Arr out[9])
	{
		out[0] = &RlcAccess::v_RLC_ilv; out[1] = &RlcAccess::v_RLC_i2v; out[2] = &RlcAccess::v_RLC_vv2;
		out[3] = &RlcAccess::v_RLC_vj1; out[4] = &RlcAccess::v_RLC_vj2; out[5] = &RlcAccess::v_RLC_vvd;
		out[6] = &RlcAccess::v_RLC_ib0; out[7] = &RlcAccess::v_RLC_b1; out[8] = &RlcAccess::v_RLC_b2;
	}
};

} // namespace

Operator_CUDA* Operator_CUDA::New()
{
	std::cout << "Create FDTD operator (GB300 CUDA engine)" << std::endl;
	Operator_CUDA* op = new Operator_CUDA();
	op->Init();
	return op;
}

Operator_CUDA::Operator_CUDA() : Operator()
{
}

Operator_CUDA::~Operator_CUDA()
{
}

Engine* Operator_CUDA::CreateEngine()
{
	m_Engine = Engine_CUDA::New(this);
	return m_Engine;
}

bool Operator_CUDA::Describe(wipems_openems::OperatorView& view) const
{
	const uint32_t n[3] = {numLines[0], numLines[1], numLines[2]};
	view.set_main(vv, vi, ii, iv, n, dT, discLines, gridDelta);
	const Operator_Ext_Excitation* exc_ext = 0;
	for (size_t k = 0; k < m_Op_exts.size(); ++k)
	{
		Operator_Extension* ext = m_Op_exts.at(k);
		if (Operator_Ext_UPML* u = dynamic_cast<Operator_Ext_UPML*>(ext))
		{
			const unsigned int* st = u->*UpmlAccess::start_();
			const unsigned int* nl = u->*UpmlAccess::lines_();
			const uint32_t s32[3] = {st[0], st[1], st[2]}, n32[3] = {nl[0], nl[1], nl[2]};
			view.add_upml(s32, n32, u->*UpmlAccess::vv_(), u->*UpmlAccess::vvfo_(), u->*UpmlAccess::vvfn_(),
						  u->*UpmlAccess::ii_(), u->*UpmlAccess::iifo_(), u->*UpmlAccess::iifn_());
		}
		else if (Operator_Ext_LorentzMaterial* l = dynamic_cast<Operator_Ext_LorentzMaterial*>(ext))
		{
			const int order = l->*LorentzAccess::order_();
			for (int o = 0; o < order; ++o)
			{
				const bool von = (l->*LorentzAccess::volt_on_())[o], con = (l->*LorentzAccess::curr_on_())[o];
				const bool vlon = (l->*LorentzAccess::volt_lor_on_())[o], clon = (l->*LorentzAccess::curr_lor_on_())[o];
				view.add_ade_order((l->*LorentzAccess::count_()).at(o), (l->*LorentzAccess::pos_())[o], von, con, vlon,
								   clon, von ? (l->*LorentzAccess::v_int_())[o] : (FDTD_FLOAT**)0,
								   von ? (l->*LorentzAccess::v_ext_())[o] : (FDTD_FLOAT**)0,
								   vlon ? (l->*LorentzAccess::v_lor_())[o] : (FDTD_FLOAT**)0,
								   con ? (l->*LorentzAccess::i_int_())[o] : (FDTD_FLOAT**)0,
								   con ? (l->*LorentzAccess::i_ext_())[o] : (FDTD_FLOAT**)0,
								   clon ? (l->*LorentzAccess::i_lor_())[o] : (FDTD_FLOAT**)0);
			}
		}
		else if (Operator_Ext_Excitation* e = dynamic_cast<Operator_Ext_Excitation*>(ext))
		{
			exc_ext = e;
			view.set_excitation(false, e->*ExcitationAccess::volt_count_(), e->*ExcitationAccess::volt_index_(),
								e->*ExcitationAccess::volt_dir_(), e->*ExcitationAccess::volt_amp_(),
								e->*ExcitationAccess::volt_delay_());
			view.set_excitation(true, e->*ExcitationAccess::curr_count_(), e->*ExcitationAccess::curr_index_(),
								e->*ExcitationAccess::curr_dir_(), e->*ExcitationAccess::curr_amp_(),
								e->*ExcitationAccess::curr_delay_());
		}
		else if (dynamic_cast<Operator_Ext_Mur_ABC*>(ext))
		{
			// below: a face's start timestep needs the excitation lists
		}
		else if (Operator_Ext_LumpedRLC* r = dynamic_cast<Operator_Ext_LumpedRLC*>(ext))
		{
			RlcAccess::Arr c[9];
			RlcAccess::coefs(c);
			FDTD_FLOAT* coef[9];
			for (int k2 = 0; k2 < 9; ++k2)
				coef[k2] = r->*c[k2];
			const unsigned int cnt = r->*RlcAccess::count_();
			if (cnt)
				view.set_rlc(cnt, r->*RlcAccess::pos_(), r->*RlcAccess::dir_(), coef);
		}
		else
		{
			std::cerr << "Operator_CUDA::Describe: the GB300 engine does not provide the extension \""
					  << ext->GetExtensionName() << "\"" << std::endl;
			return false;
		}
	}
	// Mur faces, with the start timestep Engine_Ext_Mur_ABC's constructor
	// derives from an excitation on the face (engine_ext_mur_abc.cpp:43-58)
	for (size_t k = 0; k < m_Op_exts.size(); ++k)
	{
		Operator_Ext_Mur_ABC* m = dynamic_cast<Operator_Ext_Mur_ABC*>(m_Op_exts.at(k));
		if (!m)
			continue;
		const int ny = m->*MurAccess::ny_(), nyP = m->*MurAccess::nyP_(), nyPP = m->*MurAccess::nyPP_();
		const unsigned int line = m->*MurAccess::line_();
		int maxDelay = -1;
		if (exc_ext)
		{
			const unsigned int cnt = exc_ext->*ExcitationAccess::volt_count_();
			const unsigned short* dir = exc_ext->*ExcitationAccess::volt_dir_();
			unsigned int* const* idx = exc_ext->*ExcitationAccess::volt_index_();
			const unsigned int* delay = exc_ext->*ExcitationAccess::volt_delay_();
			for (unsigned int i = 0; i < cnt; ++i)
				if (((dir[i] == nyP) || (dir[i] == nyPP)) && (idx[ny][i] == line) && ((int)delay[i] > maxDelay))
					maxDelay = (int)delay[i];
		}
		const uint32_t start_ts = maxDelay >= 0 ? (uint32_t)maxDelay + m_Exc->GetLength() + 10 : 0;
		const unsigned int* nl = m->*MurAccess::lines_();
		view.add_mur(ny, m->*MurAccess::top_(), line, (uint32_t)(m->*MurAccess::shift_()), nl[0], nl[1],
					 m->*MurAccess::coef_p_(), m->*MurAccess::coef_pp_(), start_ts);
	}
	// Engine_Ext_Excitation's period in timesteps (engine_ext_excitation.cpp:44-46)
	const double period = m_Exc->GetSignalPeriod();
	view.set_signal(m_Exc->GetVoltageSignal(), m_Exc->GetCurrentSignal(), m_Exc->GetLength(),
					period > 0 ? (uint32_t)(period / dT) : 0u);
	view.finish();
	return true;
}
