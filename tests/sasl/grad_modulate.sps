// tex2D (the sampler's sample_2d_grad with the coordinate's quad
// differences) modulated by the interpolated colour.
sampler s;

struct PSIn {
	float4 uv:    TEXCOORD0;
	float4 color: COLOR0;
};

float4 ps_main(PSIn in): COLOR {
	return tex2D(s, in.uv.xy) * in.color;
}
