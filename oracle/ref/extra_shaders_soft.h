/*
 * Test infrastructure (checker only): software shaders that the synthetic benchmark scenes need
 * and that the reference does not ship. They are ShaderSoft subclasses, so they run under the
 * unmodified reference RendererSoft exactly like the reference's own shaders
 * (src/Viewer/Shader/Software/*.h), loaded the way ViewerSoftware::loadShaders does
 * (src/Viewer/ViewerSoftware.h:54-69).
 *
 *  - ShaderBlinnPhongDir: Blinn-Phong with one directional light and shininess 32. It reuses the
 *    reference's Blinn-Phong interface structs, normal mapping and 3x3 PCF shadow lookup
 *    (BlinnPhongSoft.h:96-271); the light uniform u_pointLightPosition carries the direction
 *    towards the light, and there is no range attenuation.
 *  - ShaderVertexColor: position + RGBA vertex colour, colour passed through unchanged.
 */
#pragma once

#include "Viewer/Shader/Software/BlinnPhongSoft.h"

namespace SoftGL {
namespace ShaderBlinnPhongDir {

using ShaderBlinnPhong::ShaderDefines;
using ShaderBlinnPhong::ShaderAttributes;
using ShaderBlinnPhong::ShaderUniforms;
using ShaderBlinnPhong::ShaderVaryings;

class VS : public ShaderBlinnPhong::VS {
 public:
  CREATE_SHADER_CLONE(VS)

  void shaderMain() override {
    SoftGL::ShaderBlinnPhong::VS::shaderMain();
    v->v_lightDirection = u->u_pointLightPosition;
  }
};

class FS : public ShaderBlinnPhong::FS {
 public:
  CREATE_SHADER_CLONE(FS)

  void shaderMain() override {
    const float specularExponent = 32.f;

    glm::vec4 baseColor;
    if (def->ALBEDO_MAP) {
      baseColor = texture(u->u_albedoMap, v->v_texCoord);
    } else {
      baseColor = u->u_baseColor;
    }

    glm::vec3 N = GetNormalFromMap();

    float ao = 1.f;
    if (def->AO_MAP) {
      ao = texture(u->u_aoMap, v->v_texCoord).r;
    }
    glm::vec3 ambientColor = glm::vec3(baseColor) * u->u_ambientColor * ao;
    glm::vec3 diffuseColor = glm::vec3(0.f);
    glm::vec3 specularColor = glm::vec3(0.f);
    glm::vec3 emissiveColor = glm::vec3(0.f);

    if (u->u_enableLight) {
      glm::vec3 lightDirection = normalize(v->v_lightDirection);
      float diffuse = glm::max(dot(N, lightDirection), 0.0f);
      diffuseColor = u->u_pointLightColor * glm::vec3(baseColor) * diffuse;

      glm::vec3 cameraDirection = normalize(v->v_cameraDirection);
      glm::vec3 halfVector = normalize(lightDirection + cameraDirection);
      float specularAngle = glm::max(dot(N, halfVector), 0.0f);
      specularColor = u->u_kSpecular * glm::vec3(glm::pow(specularAngle, specularExponent));

      if (u->u_enableShadow) {
        float shadow = 1.0f - ShadowCalculation(v->v_shadowFragPos, N);
        diffuseColor *= shadow;
        specularColor *= shadow;
      }
    }

    if (def->EMISSIVE_MAP) {
      emissiveColor = texture(u->u_emissiveMap, v->v_texCoord);
    }

    gl->FragColor = glm::vec4(ambientColor + diffuseColor + specularColor + emissiveColor, baseColor.a);
  }
};

}  // namespace ShaderBlinnPhongDir

namespace ShaderVertexColor {

struct ShaderDefines {
};

struct ShaderAttributes {
  glm::vec3 a_position;
  glm::vec4 a_color;
};

struct ShaderUniforms {
  // UniformsModel
  glm::int32_t u_reverseZ;
  glm::mat4 u_modelMatrix;
  glm::mat4 u_modelViewProjectionMatrix;
  glm::mat3 u_inverseTransposeModelMatrix;
  glm::mat4 u_shadowMVPMatrix;

  // UniformsMaterial
  glm::int32_t u_enableLight;
  glm::int32_t u_enableIBL;
  glm::int32_t u_enableShadow;
  glm::float32_t u_pointSize;
  glm::float32_t u_kSpecular;
  glm::vec4 u_baseColor;
};

struct ShaderVaryings {
  glm::vec4 v_color;
};

class ShaderVertexColor : public ShaderSoft {
 public:
  CREATE_SHADER_OVERRIDE

  std::vector<std::string> &getDefines() override {
    static std::vector<std::string> defines;
    return defines;
  }

  std::vector<UniformDesc> &getUniformsDesc() override {
    static std::vector<UniformDesc> desc = {
        {"UniformsModel", offsetof(ShaderUniforms, u_reverseZ)},
        {"UniformsMaterial", offsetof(ShaderUniforms, u_enableLight)},
    };
    return desc;
  };
};

class VS : public ShaderVertexColor {
 public:
  CREATE_SHADER_CLONE(VS)

  void shaderMain() override {
    gl->Position = u->u_modelViewProjectionMatrix * glm::vec4(a->a_position, 1.0);
    v->v_color = a->a_color;
  }
};

class FS : public ShaderVertexColor {
 public:
  CREATE_SHADER_CLONE(FS)

  void shaderMain() override {
    gl->FragColor = v->v_color;
  }
};

}  // namespace ShaderVertexColor
}  // namespace SoftGL
